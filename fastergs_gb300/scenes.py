"""Seeded synthetic scenes and cameras for tests and benchmarks.

The reference is evaluated on Mip-NeRF 360 / Tanks & Temples / Deep Blending
scenes, which are not available here; these generators produce seeded
stand-ins with the Gaussian counts, resolutions and parameter distributions
of the benchmark configurations:

  c1   10,000 Gaussians, 256x256, 60 deg FoV, SH degree 0 (CPU-oracle size)
  c2   1,000,000 Gaussians in a 10x10x10 box 2-12 units ahead, 1297x840,
       50 deg FoV, heavy-tailed log-scales N(-4, 1), SH degree 3
  c3   3,000,000 Gaussians from 64 anisotropic clusters with Zipf(1.2)
       weights, log-scales N(-5, 1.2), SH degree 3, 1920x1080
  c4   the c2 scene seen by 16 cameras on a radius-8 circle, mixed resolutions
  c5a  2,000 Gaussians, 128x128, SH degree 1 (finite-difference checks)
  c5b  6,000,000 Gaussians, c3 distribution, 3840x2160

Cameras follow the 3DGS conventions (x right, y down, z forward): the view
matrix is getWorld2View2(R, T) transposed and the full projection is
view @ getProjectionMatrix(...)^T, both stored row-major as the kernels read
them (3DGS/scene/cameras.py:54-57, 3DGS/utils/graphics_utils.py:38-71).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def projection_matrix(znear: float, zfar: float, fovx: float, fovy: float) -> np.ndarray:
    """Perspective matrix of 3DGS/utils/graphics_utils.py:51-71 (row-major, not transposed)."""
    top = math.tan(fovy / 2) * znear
    right = math.tan(fovx / 2) * znear
    bottom, left = -top, -right
    P = np.zeros((4, 4), dtype=np.float64)
    P[0, 0] = 2.0 * znear / (right - left)
    P[1, 1] = 2.0 * znear / (top - bottom)
    P[0, 2] = (right + left) / (right - left)
    P[1, 2] = (top + bottom) / (top - bottom)
    P[3, 2] = 1.0
    P[2, 2] = zfar / (zfar - znear)
    P[2, 3] = -(zfar * znear) / (zfar - znear)
    return P


def world_to_view(R: np.ndarray, t: np.ndarray) -> np.ndarray:
    """getWorld2View2 with no extra translation or scale: [R^T | t]."""
    Rt = np.zeros((4, 4), dtype=np.float64)
    Rt[:3, :3] = R.T
    Rt[:3, 3] = t
    Rt[3, 3] = 1.0
    return Rt


def look_at(eye, target, down=(0.0, 1.0, 0.0)):
    """Camera-to-world rotation R (columns = camera x, y, z in world) and the
    world-to-view translation t for a camera at eye looking at target."""
    eye = np.asarray(eye, dtype=np.float64)
    z = np.asarray(target, dtype=np.float64) - eye
    z /= np.linalg.norm(z)
    x = np.cross(np.asarray(down, dtype=np.float64), z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    R = np.stack([x, y, z], axis=1)
    t = -R.T @ eye
    return R, t


@dataclass
class Camera:
    width: int
    height: int
    fovx: float
    fovy: float
    viewmatrix: np.ndarray     # (4,4) float32, world_view_transform
    projmatrix: np.ndarray     # (4,4) float32, full_proj_transform
    campos: np.ndarray         # (3,) float32
    znear: float = 0.01
    zfar: float = 100.0

    @property
    def tanfovx(self) -> float:
        return math.tan(self.fovx * 0.5)

    @property
    def tanfovy(self) -> float:
        return math.tan(self.fovy * 0.5)


def make_camera(width: int, height: int, fovx_deg: float, eye=(0.0, 0.0, 0.0), target=(0.0, 0.0, 1.0),
                znear: float = 0.01, zfar: float = 100.0, fovy_deg: float | None = None) -> Camera:
    fovx = math.radians(fovx_deg)
    if fovy_deg is None:  # square pixels: same focal length on both axes
        fovy = 2.0 * math.atan(math.tan(fovx / 2) * height / width)
    else:
        fovy = math.radians(fovy_deg)
    R, t = look_at(eye, target)
    w2v = world_to_view(R, t).astype(np.float32)
    world_view = w2v.T.copy()
    proj = projection_matrix(znear, zfar, fovx, fovy).astype(np.float32).T.copy()
    full = (world_view.astype(np.float64) @ proj.astype(np.float64)).astype(np.float32)
    campos = np.linalg.inv(world_view.astype(np.float64))[3, :3].astype(np.float32)
    return Camera(width, height, fovx, fovy, world_view, full, campos, znear, zfar)


@dataclass
class Scene:
    """Raw (pre-activation) Gaussian parameters, float32."""
    means: np.ndarray          # (P,3)
    log_scales: np.ndarray     # (P,3)
    quats: np.ndarray          # (P,4) raw (r,x,y,z)
    opacity_logits: np.ndarray # (P,1)
    dc: np.ndarray             # (P,1,3)
    shs: np.ndarray            # (P,15,3)
    sh_degree: int
    camera: Camera
    name: str = ""

    @property
    def P(self) -> int:
        return self.means.shape[0]

    def activated(self):
        """(means, scales, rotations, opacities, dc, shs) as the rasterizer takes them."""
        q = self.quats.astype(np.float64)
        q = q / np.linalg.norm(q, axis=1, keepdims=True)
        return (self.means, np.exp(self.log_scales.astype(np.float64)).astype(np.float32), q.astype(np.float32),
                (1.0 / (1.0 + np.exp(-self.opacity_logits.astype(np.float64)))).astype(np.float32), self.dc,
                self.shs)


def _sh(rng, P, degree, dc_std, rest_std):
    dc = rng.normal(0.0, dc_std, size=(P, 1, 3)).astype(np.float32)
    shs = np.zeros((P, 15, 3), dtype=np.float32)
    used = (degree + 1) ** 2 - 1
    if used:
        shs[:, :used] = rng.normal(0.0, rest_std, size=(P, used, 3))
    return dc, shs


def scene_c1(seed: int = 0, P: int = 10_000) -> Scene:
    rng = np.random.default_rng(seed)
    means = rng.normal(0.0, 1.0, size=(P, 3)) + np.array([0.0, 0.0, 4.0])
    log_scales = rng.normal(-4.5, 0.5, size=(P, 3))
    quats = rng.normal(0.0, 1.0, size=(P, 4))
    logits = rng.normal(0.0, 1.0, size=(P, 1))
    dc, shs = _sh(rng, P, 0, 0.3, 0.0)
    cam = make_camera(256, 256, 60.0, fovy_deg=60.0)
    return Scene(means.astype(np.float32), log_scales.astype(np.float32), quats.astype(np.float32),
                 logits.astype(np.float32), dc, shs, 0, cam, "c1")


def scene_c2(seed: int = 0, P: int = 1_000_000, width: int = 1297, height: int = 840) -> Scene:
    rng = np.random.default_rng(seed)
    means = np.stack([rng.uniform(-5, 5, P), rng.uniform(-5, 5, P), rng.uniform(2, 12, P)], axis=1)
    log_scales = rng.normal(-4.0, 1.0, size=(P, 3))
    quats = rng.normal(0.0, 1.0, size=(P, 4))
    logits = rng.normal(0.0, 1.5, size=(P, 1))
    dc, shs = _sh(rng, P, 3, 0.5, 0.2)
    cam = make_camera(width, height, 50.0)
    return Scene(means.astype(np.float32), log_scales.astype(np.float32), quats.astype(np.float32),
                 logits.astype(np.float32), dc, shs, 3, cam, "c2")


def _random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    r, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)], -1),
        np.stack([2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)], -1),
        np.stack([2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], -1)], axis=1)


def scene_clusters(seed: int, P: int, width: int, height: int, name: str) -> Scene:
    rng = np.random.default_rng(seed)
    K = 64
    centers = np.stack([rng.uniform(-10, 10, K), rng.uniform(-10, 10, K), rng.uniform(2, 22, K)], axis=1)
    axes = np.exp(rng.uniform(math.log(0.05), math.log(3.0), size=(K, 3)))
    rots = _random_rotations(rng, K)
    w = 1.0 / np.arange(1, K + 1) ** 1.2
    w /= w.sum()
    cid = rng.choice(K, size=P, p=w)
    local = rng.normal(size=(P, 3)) * axes[cid]
    means = centers[cid] + np.einsum("pij,pj->pi", rots[cid], local)
    log_scales = rng.normal(-5.0, 1.2, size=(P, 3))
    quats = rng.normal(0.0, 1.0, size=(P, 4))
    logits = rng.normal(0.0, 2.0, size=(P, 1))
    dc, shs = _sh(rng, P, 3, 0.5, 0.2)
    cam = make_camera(width, height, 60.0)
    return Scene(means.astype(np.float32), log_scales.astype(np.float32), quats.astype(np.float32),
                 logits.astype(np.float32), dc, shs, 3, cam, name)


def scene_c3(seed: int = 0, P: int = 3_000_000) -> Scene:
    return scene_clusters(seed, P, 1920, 1080, "c3")


def scene_c5b(seed: int = 0, P: int = 6_000_000) -> Scene:
    return scene_clusters(seed, P, 3840, 2160, "c5b")


C4_RESOLUTIONS = [(640, 360), (960, 540), (1297, 840), (1600, 900), (1920, 1080)]


def cameras_c4(seed: int = 0, n: int = 16, radius: float = 8.0, center=(0.0, 0.0, 7.0)) -> list[Camera]:
    rng = np.random.default_rng(seed + 1000)
    cams = []
    for k in range(n):
        th = 2 * math.pi * k / n
        eye = (center[0] + radius * math.sin(th), center[1], center[2] - radius * math.cos(th))
        w, h = C4_RESOLUTIONS[int(rng.integers(len(C4_RESOLUTIONS)))]
        cams.append(make_camera(w, h, float(rng.uniform(40.0, 70.0)), eye=eye, target=center))
    return cams


def scene_c5a(seed: int = 0, P: int = 2_000) -> Scene:
    rng = np.random.default_rng(seed)
    means = rng.normal(0.0, 1.0, size=(P, 3)) + np.array([0.0, 0.0, 4.0])
    log_scales = rng.normal(-3.5, 0.5, size=(P, 3))
    quats = rng.normal(0.0, 1.0, size=(P, 4))
    logits = rng.normal(0.0, 1.0, size=(P, 1))
    dc, shs = _sh(rng, P, 1, 0.3, 0.2)
    cam = make_camera(128, 128, 60.0, fovy_deg=60.0)
    return Scene(means.astype(np.float32), log_scales.astype(np.float32), quats.astype(np.float32),
                 logits.astype(np.float32), dc, shs, 1, cam, "c5a")


def upstream_grad(seed: int, height: int, width: int) -> np.ndarray:
    """dL/dimage ~ N(0, 1), shape (3, H, W), float32."""
    return np.random.default_rng(seed + 7).normal(size=(3, height, width)).astype(np.float32)
