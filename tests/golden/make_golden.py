"""Generates the golden fixtures that pin the CPU oracle against the reference.

Runs the reference's own Python code, imported from the FasterGS checkout
named by the FASTERGS_REF environment variable (required), on seeded inputs and
stores inputs and outputs in tests/golden/*.npz:

  sh_golden.npz       3DGS/utils/sh_utils.py eval_sh, degrees 0..3
  cov_golden.npz      3DGS/utils/general_utils.py build_scaling_rotation ->
                      L L^T -> strip_symmetric (the 3DGS covariance path)
  camera_golden.npz   3DGS/utils/graphics_utils.py getWorld2View2 /
                      getProjectionMatrix composed as 3DGS/scene/cameras.py:54-57
  ply_golden.npz      3DGS/scene/gaussian_model.py save_ply (the vertex array it
                      hands plyfile: property names and values) and load_ply
                      (the tensors it builds from that array), SH degrees 1, 3
  camera_ts_golden.npz  getWorld2View2 with a translate / scale, composed as
                      3DGS/scene/cameras.py:54-57
  ssim_golden.npz     3DGS/utils/loss_utils.py ssim (per-image means) and the
                      training loss (1 - lambda) l1_loss + lambda (1 - ssim),
                      with their gradients w.r.t. the rendered image by
                      autograd, in FP64 (the window is the module's own)

build_rotation / build_scaling_rotation allocate with device='cuda'; the
script runs them on CPU by handing the module a torch proxy whose zeros()
(and, for load_ply, tensor()) drops the device argument.  gaussian_model.py
imports plyfile and simple_knn, absent here: it gets stand-ins whose PlyData /
PlyElement capture the array save_ply writes and hand it back to load_ply.
Nothing else of the reference is changed.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib.util
import math
import os
import sys
import types
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent


def _ref() -> Path:
    """The FasterGS checkout whose Python code generates the fixtures (FASTERGS_REF, required)."""
    ref = os.environ.get("FASTERGS_REF")
    if not ref:
        raise SystemExit("set FASTERGS_REF to the FasterGS checkout (its 3DGS/ Python code makes the fixtures)")
    return Path(ref)


def _load(rel: str, name: str):
    spec = importlib.util.spec_from_file_location(name, _ref() / rel)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _cpu_torch_proxy():
    proxy = types.SimpleNamespace(**{k: getattr(torch, k) for k in dir(torch) if not k.startswith("__")})

    def zeros(*args, **kwargs):
        kwargs.pop("device", None)
        return torch.zeros(*args, **kwargs)

    proxy.zeros = zeros
    return proxy


def make_sh(rng):
    sh_utils = _load("3DGS/utils/sh_utils.py", "ref_sh_utils")
    n = 512
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    coeffs = rng.normal(size=(n, 16, 3))  # (n, k, channel)
    out = {}
    for deg in range(4):
        sh = torch.tensor(coeffs, dtype=torch.float64).transpose(1, 2)  # (n, 3, 16) as eval_sh wants
        out[f"deg{deg}"] = sh_utils.eval_sh(deg, sh, torch.tensor(dirs, dtype=torch.float64)).numpy()
    np.savez_compressed(HERE / "sh_golden.npz", dirs=dirs, coeffs=coeffs, **out)


def make_cov(rng):
    gu = _load("3DGS/utils/general_utils.py", "ref_general_utils")
    gu.torch = _cpu_torch_proxy()
    n = 512
    scales = np.exp(rng.normal(-2.0, 1.0, size=(n, 3)))
    quats = rng.normal(size=(n, 4))
    quats /= np.linalg.norm(quats, axis=1, keepdims=True)
    L = gu.build_scaling_rotation(torch.tensor(scales, dtype=torch.float32), torch.tensor(quats, dtype=torch.float32))
    cov = gu.strip_symmetric(L @ L.transpose(1, 2))
    np.savez_compressed(HERE / "cov_golden.npz", scales=scales, quats=quats, cov=cov.numpy().astype(np.float64))


def make_cameras(rng):
    gr = _load("3DGS/utils/graphics_utils.py", "ref_graphics_utils")
    cases = []
    for k in range(6):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        r, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)],
                      [2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)],
                      [2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)]])
        T = rng.normal(size=3) * 3
        fovx = math.radians(float(rng.uniform(40, 80)))
        fovy = math.radians(float(rng.uniform(30, 70)))
        wv = torch.tensor(gr.getWorld2View2(R, T)).transpose(0, 1)
        pm = gr.getProjectionMatrix(znear=0.01, zfar=100.0, fovX=fovx, fovY=fovy).transpose(0, 1)
        full = wv.unsqueeze(0).bmm(pm.unsqueeze(0)).squeeze(0)
        center = wv.inverse()[3, :3]
        cases.append((R, T, fovx, fovy, wv.numpy(), pm.numpy(), full.numpy(), center.numpy()))
    arr = lambda i: np.stack([c[i] for c in cases])
    np.savez_compressed(HERE / "camera_golden.npz", R=arr(0), T=arr(1), fovx=arr(2), fovy=arr(3),
                        world_view=arr(4), proj=arr(5), full_proj=arr(6), center=arr(7))


def make_ssim(rng):
    lu = _load("3DGS/utils/loss_utils.py", "ref_loss_utils")
    out = {}
    for k, (B, C, H, W) in enumerate([(1, 3, 37, 53), (2, 1, 64, 40)]):
        img = rng.uniform(0.0, 1.0, size=(B, C, H, W))
        gt = np.clip(img + rng.normal(0.0, 0.15, size=img.shape), 0.0, 1.0)
        x = torch.tensor(img, dtype=torch.float64, requires_grad=True)
        y = torch.tensor(gt, dtype=torch.float64)
        per_image = lu.ssim(x, y, size_average=False)          # mean SSIM per image
        g_ssim, = torch.autograd.grad(per_image.sum(), x)      # d sum of image means / d img
        x2 = torch.tensor(img, dtype=torch.float64, requires_grad=True)
        lam = 0.2
        loss = (1.0 - lam) * lu.l1_loss(x2, y) + lam * (1.0 - lu.ssim(x2, y))
        g_loss, = torch.autograd.grad(loss, x2)
        out.update({f"img{k}": img, f"gt{k}": gt, f"ssim{k}": per_image.detach().numpy(),
                    f"grad_ssim{k}": g_ssim.numpy(), f"loss{k}": np.float64(loss.item()),
                    f"grad_loss{k}": g_loss.numpy()})
    out["lam"] = np.float64(0.2)
    np.savez_compressed(HERE / "ssim_golden.npz", **out)


class _PlyCapture:
    """Stand-in for the plyfile module: keeps the vertex array save_ply describes."""

    def __init__(self):
        self.elements = None
        cap = self

        class PlyElement:
            @staticmethod
            def describe(arr, name):
                return (name, arr)

        class _Props:
            def __init__(self, name):
                self.name = name

        class _Element:
            def __init__(self, arr):
                self.arr = arr
                self.properties = [_Props(n) for n in arr.dtype.names]

            def __getitem__(self, k):
                return self.arr[k]

        class PlyData:
            def __init__(self, els=None):
                self.els = els or []
                self.elements = [_Element(a) for _, a in self.els]

            def write(self, path):
                cap.elements = self.els

            @staticmethod
            def read(path):
                return PlyData(cap.elements)

        self.module = types.SimpleNamespace(PlyData=PlyData, PlyElement=PlyElement)


def make_ply(rng):
    import tempfile
    cap = _PlyCapture()
    saved = {k: sys.modules.get(k) for k in ("plyfile", "simple_knn", "simple_knn._C")}
    sys.modules["plyfile"] = cap.module
    sys.modules["simple_knn"] = types.ModuleType("simple_knn")
    sys.modules["simple_knn._C"] = types.SimpleNamespace(distCUDA2=None)
    sys.path.insert(0, str(_ref() / "3DGS"))
    try:
        gm = _load("3DGS/scene/gaussian_model.py", "ref_gaussian_model")
        proxy = _cpu_torch_proxy()
        tensor = torch.tensor

        def tensor_cpu(*args, **kwargs):
            kwargs.pop("device", None)
            return tensor(*args, **kwargs)

        proxy.tensor = tensor_cpu
        gm.torch = proxy
        out = {}
        for deg in (1, 3):
            P, M = 37, (deg + 1) ** 2 - 1
            model = object.__new__(gm.GaussianModel)
            model.max_sh_degree = deg
            f = lambda *shape: torch.tensor(rng.normal(size=shape), dtype=torch.float32)
            model._xyz, model._features_dc, model._features_rest = f(P, 3), f(P, 1, 3), f(P, M, 3)
            model._opacity, model._scaling, model._rotation = f(P, 1), f(P, 3), f(P, 4)
            with tempfile.TemporaryDirectory() as d:
                model.save_ply(os.path.join(d, "point_cloud.ply"))
                (_, arr), = cap.elements
                loaded = object.__new__(gm.GaussianModel)
                loaded.max_sh_degree = deg
                loaded.load_ply(os.path.join(d, "point_cloud.ply"))
            out[f"names{deg}"] = np.array(arr.dtype.names)
            out[f"vertex{deg}"] = np.stack([arr[n] for n in arr.dtype.names], axis=1).astype(np.float32)
            for k, t in (("xyz", model._xyz), ("f_dc", model._features_dc), ("f_rest", model._features_rest),
                         ("opacity", model._opacity), ("scaling", model._scaling), ("rotation", model._rotation)):
                out[f"{k}{deg}"] = t.numpy()
            for k, t in (("xyz", loaded._xyz), ("f_dc", loaded._features_dc), ("f_rest", loaded._features_rest),
                         ("opacity", loaded._opacity), ("scaling", loaded._scaling),
                         ("rotation", loaded._rotation)):
                out[f"loaded_{k}{deg}"] = t.detach().numpy()
        np.savez_compressed(HERE / "ply_golden.npz", **out)
    finally:
        sys.path.remove(str(_ref() / "3DGS"))
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


def make_cameras_ts(rng):
    gr = _load("3DGS/utils/graphics_utils.py", "ref_graphics_utils_ts")
    out = {k: [] for k in ("R", "T", "translate", "scale", "fovx", "fovy", "world_view", "full_proj", "center")}
    for k in range(4):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        r, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)],
                      [2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)],
                      [2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)]])
        T = rng.normal(size=3) * 2
        tr = rng.normal(size=3)
        sc = float(rng.uniform(0.5, 2.0))
        fovx = math.radians(float(rng.uniform(40, 80)))
        fovy = math.radians(float(rng.uniform(30, 70)))
        wv = torch.tensor(gr.getWorld2View2(R, T, tr, sc)).transpose(0, 1)
        pm = gr.getProjectionMatrix(znear=0.01, zfar=100.0, fovX=fovx, fovY=fovy).transpose(0, 1)
        full = wv.unsqueeze(0).bmm(pm.unsqueeze(0)).squeeze(0)
        for key, val in (("R", R), ("T", T), ("translate", tr), ("scale", sc), ("fovx", fovx), ("fovy", fovy),
                         ("world_view", wv.numpy()), ("full_proj", full.numpy()),
                         ("center", wv.inverse()[3, :3].numpy())):
            out[key].append(val)
    np.savez_compressed(HERE / "camera_ts_golden.npz", **{k: np.stack(v) for k, v in out.items()})


def main():
    if not _ref().exists():
        sys.exit(f"reference checkout not found at {_ref()}")
    rng = np.random.default_rng(20240611)
    make_sh(rng)
    make_cov(rng)
    make_cameras(rng)
    make_ssim(np.random.default_rng(20241204))
    make_ply(np.random.default_rng(7))
    make_cameras_ts(np.random.default_rng(8))
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
