"""Camera construction as FasterGS's backbones build it, and the rasterizer
settings of a render call.

``camera_from_rt`` follows 3DGS/scene/cameras.py:54-57 with
utils/graphics_utils.py getWorld2View2 (:38-49) and getProjectionMatrix
(:51-71): world_view = getWorld2View2(R, T, translate, scale)^T, proj =
getProjectionMatrix(znear, zfar, FoVx, FoVy)^T, full_proj = world_view @ proj,
camera centre = inverse(world_view)[3, :3].  ``raster_settings`` fills
GaussianRasterizationSettings as gaussian_renderer/render_faster.py:28-43
does.
"""
from __future__ import annotations

import math

import numpy as np

from .scenes import Camera, projection_matrix


def world_to_view(R, T, translate=(0.0, 0.0, 0.0), scale: float = 1.0) -> np.ndarray:
    """getWorld2View2: [R^T | T] with the camera centre moved by translate and scaled (float32)."""
    Rt = np.zeros((4, 4))
    Rt[:3, :3] = np.asarray(R, np.float64).T
    Rt[:3, 3] = np.asarray(T, np.float64)
    Rt[3, 3] = 1.0
    C2W = np.linalg.inv(Rt)
    C2W[:3, 3] = (C2W[:3, 3] + np.asarray(translate, np.float64)) * scale
    return np.float32(np.linalg.inv(C2W))


def camera_from_rt(R, T, fovx: float, fovy: float, width: int, height: int, znear: float = 0.01,
                   zfar: float = 100.0, translate=(0.0, 0.0, 0.0), scale: float = 1.0) -> Camera:
    """A camera from a COLMAP-style rotation R (camera-to-world, as 3DGS stores it), translation T
    (world-to-view) and field of view in radians."""
    world_view = world_to_view(R, T, translate, scale).T.copy()
    proj = projection_matrix(znear, zfar, fovx, fovy).astype(np.float32).T.copy()
    full = (world_view.astype(np.float64) @ proj.astype(np.float64)).astype(np.float32)
    campos = np.linalg.inv(world_view.astype(np.float64))[3, :3].astype(np.float32)
    return Camera(int(width), int(height), float(fovx), float(fovy), world_view, full, campos, znear, zfar)


def raster_settings(cam: Camera, bg=(0.0, 0.0, 0.0), sh_degree: int = 3, scale_modifier: float = 1.0,
                    mult: float = 1.0, device="cuda", debug: bool = False):
    """GaussianRasterizationSettings for one render of cam (render_faster.py:28-43)."""
    import torch
    from . import GaussianRasterizationSettings
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=device)
    return GaussianRasterizationSettings(
        image_height=int(cam.height), image_width=int(cam.width), tanfovx=math.tan(cam.fovx * 0.5),
        tanfovy=math.tan(cam.fovy * 0.5), bg=t(bg), scale_modifier=scale_modifier, viewmatrix=t(cam.viewmatrix),
        projmatrix=t(cam.projmatrix), sh_degree=sh_degree, campos=t(cam.campos), mult=mult, prefiltered=False,
        debug=debug)
