"""FP64 CPU oracle of the FasterGS rasterizer -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker or the timed CPU
baseline.  The product (``fastergs_gb300``) never calls it.

Parity status: pinned.  SH evaluation, scale/rotation covariance and camera
matrices against the reference's own Python code (fixtures under
tests/golden/); the rasterizer core, a restatement of the reference CUDA
source (oracle.cpp holds the file:line map), against the outputs of the
reference CUDA backend built for sm_103a and run on a GB300
(tests/golden/fb_*.npz, made by tests/golden/make_fb_golden.py).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import platform
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.cpp"
LIB = HERE / "liboracle.so"
STAMP = HERE / "liboracle.so.stamp"

_lib = None


def _stamp() -> str:
    return hashlib.sha256(SRC.read_bytes() + platform.machine().encode()).hexdigest()


def build(force: bool = False) -> Path:
    """g++ -O2 -fopenmp -shared; skipped when the stamp (source hash and machine) matches."""
    if not force and LIB.exists() and STAMP.exists() and STAMP.read_text() == _stamp():
        return LIB
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    STAMP.write_text(_stamp())
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        vp, i32, i64, f64 = C.c_void_p, C.c_int, C.c_int64, C.c_double
        sig = {
            "orc_new": (vp, []),
            "orc_free": (None, [vp]),
            "orc_set_scene": (i32, [vp, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, f64, i32, i32, i32, i32, vp,
                                    vp, vp, f64, f64, f64]),
            "orc_preprocess": (None, [vp]),
            "orc_set_records": (None, [vp, vp, vp, vp]),
            "orc_emit_sort": (i64, [vp, f64]),
            "orc_set_lists": (None, [vp, i64, vp, vp]),
            "orc_render": (None, [vp, vp, i32, f64, f64]),
            "orc_num_pairs": (i64, [vp]),
            "orc_num_candidates": (i64, [vp]),
            "orc_get_candidates": (None, [vp, vp, vp]),
            "orc_num_buckets": (i64, [vp]),
            "orc_get_preprocess": (None, [vp, vp, vp, vp, vp, vp]),
            "orc_get_pairs": (None, [vp, vp, vp, vp, vp]),
            "orc_get_image": (None, [vp, vp, vp, vp, vp, vp, vp]),
            "orc_backward": (None, [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
            "orc_densify": (None, [vp, vp, vp, vp, vp, vp]),
            "orc_render_simp": (None, [vp, f64, f64, f64, vp, vp, vp, vp]),
            "orc_render_depth": (None, [vp, f64, f64, f64, vp, vp, vp, vp, vp, vp]),
            "orc_num_threads": (i32, []),
            "orc_set_threads": (None, [i32]),
            "orc_eval_sh": (None, [i32, i32, vp, vp, vp]),
            "orc_get_decisions": (None, [vp, vp, vp]),
            "orc_cov3d": (None, [i32, vp, vp, f64, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _d(a):
    """float64 C-contiguous copy (or None)."""
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One scene + camera.  Typical use: set_scene -> preprocess -> emit_sort -> render -> backward."""

    def __init__(self):
        self.lib = load()
        self.h = self.lib.orc_new()
        self._keep = []

    def __del__(self):
        if getattr(self, "h", None) and self.lib is not None:
            self.lib.orc_free(self.h)
            self.h = None

    def set_scene(self, means, opacities, scales, rotations, camera, dc=None, shs=None, colors=None, sh_degree=0,
                  culling=None, scale_modifier=1.0, mult=1.0, block=(16, 16)):
        P = means.shape[0]
        self.P, self.W, self.H = P, camera.width, camera.height
        self.bx, self.by = block
        self.gx = (self.W + self.bx - 1) // self.bx
        self.gy = (self.H + self.by - 1) // self.by
        self.M = 0 if shs is None else shs.shape[1]
        arrs = [_d(means), _d(colors), _d(dc), _d(shs), _d(opacities).reshape(-1), _d(scales), _d(rotations)]
        cull = None if culling is None else np.ascontiguousarray(np.asarray(culling, dtype=np.uint8))
        view = _d(np.asarray(camera.viewmatrix).reshape(-1))
        proj = _d(np.asarray(camera.projmatrix).reshape(-1))
        cpos = _d(camera.campos)
        self._keep = arrs + [cull, view, proj, cpos]
        st = self.lib.orc_set_scene(self.h, P, int(sh_degree), self.M, *[_p(a) for a in arrs], _p(cull),
                                    float(scale_modifier), self.W, self.H, self.bx, self.by, _p(view), _p(proj),
                                    _p(cpos), float(camera.tanfovx), float(camera.tanfovy), float(mult))
        if st != 0:
            raise ValueError("oracle rejected the scene (missing scales/rotations or colour inputs)")
        return self

    def preprocess(self):
        self.lib.orc_preprocess(self.h)
        return self

    def records(self):
        rec = np.empty((self.P, 32), np.float64)
        radii = np.empty(self.P, np.int32)
        valid = np.empty(self.P, np.uint8)
        amb = np.empty(self.P, np.uint8)
        area = np.empty(self.P, np.int32)
        self.lib.orc_get_preprocess(self.h, _p(rec), _p(radii), _p(valid), _p(amb), _p(area))
        return dict(rec=rec, radii=radii, valid=valid.astype(bool), ambiguous=amb.astype(bool), rect_area=area)

    def set_records(self, rec, radii, valid):
        rec = _d(rec)
        radii = np.ascontiguousarray(radii, dtype=np.int32)
        valid = np.ascontiguousarray(valid, dtype=np.uint8)
        self._keep_rec = (rec, radii, valid)
        self.lib.orc_set_records(self.h, _p(rec), _p(radii), _p(valid))
        return self

    def emit_sort(self, eps_pair: float = 1e-5) -> int:
        return int(self.lib.orc_emit_sort(self.h, float(eps_pair)))

    def pairs(self):
        """Sorted (key, id) lists with their ambiguity flags and tile ranges, plus the candidate-only
        pairs (``cand_keys`` / ``cand_ids``: the FP64 tile test rejects them, an FP32 evaluation of
        the same test may accept them; they are not in the lists) and ``flagged_tiles``, the tiles
        holding a flagged or candidate pair."""
        K = int(self.lib.orc_num_pairs(self.h))
        keys = np.empty(K, np.uint64)
        ids = np.empty(K, np.int32)
        amb = np.empty(K, np.uint8)
        ranges = np.empty((self.gx * self.gy, 2), np.int32)
        self.lib.orc_get_pairs(self.h, _p(keys), _p(ids), _p(amb), _p(ranges))
        Kc = int(self.lib.orc_num_candidates(self.h))
        ckeys = np.empty(Kc, np.uint64)
        cids = np.empty(Kc, np.int32)
        self.lib.orc_get_candidates(self.h, _p(ckeys), _p(cids))
        amb = amb.astype(bool)
        flagged = np.union1d(keys[amb] >> np.uint64(32), ckeys >> np.uint64(32)).astype(np.int64)
        return dict(keys=keys, ids=ids, ambiguous=amb, ranges=ranges, cand_keys=ckeys, cand_ids=cids,
                    flagged_tiles=flagged)

    def set_lists(self, ids, ranges):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        ranges = np.ascontiguousarray(ranges, dtype=np.int32).reshape(-1)
        self._keep_lists = (ids, ranges)
        self.lib.orc_set_lists(self.h, int(ids.size), _p(ids), _p(ranges))
        return self

    def render(self, bg=(0.0, 0.0, 0.0), bucket_size: int = 128, eps_alpha: float = 1e-5, eps_T: float = 1e-5):
        bgd = _d(np.asarray(bg).reshape(3))
        self.lib.orc_render(self.h, _p(bgd), int(bucket_size), float(eps_alpha), float(eps_T))
        return self

    def image(self):
        HW = self.W * self.H
        out = np.empty((3, self.H, self.W), np.float64)
        pc = np.empty((self.H, self.W, 3), np.float64)
        lc = np.empty((self.H, self.W), np.int32)
        tf = np.empty((self.H, self.W), np.float64)
        amb = np.empty((self.H, self.W), np.uint8)
        mc = np.empty(self.gx * self.gy, np.int32)
        self.lib.orc_get_image(self.h, _p(out), _p(pc), _p(lc), _p(tf), _p(amb), _p(mc))
        return dict(out_color=out, pixel_colors=pc, last_contributor=lc, Ts_final=tf, ambiguous=amb.astype(bool),
                    max_contrib=mc, num_buckets=int(self.lib.orc_num_buckets(self.h)))

    def decisions(self):
        """(#evaluations with alpha >= 1/255, #clamped at 0.99), per-Gaussian clamp flags."""
        counts = np.zeros(2, np.int64)
        cl = np.zeros(self.P, np.uint8)
        self.lib.orc_get_decisions(self.h, _p(counts), _p(cl))
        return (int(counts[0]), int(counts[1])), cl.astype(bool)

    def backward(self, dL_dout):
        P, M = self.P, self.M
        dL = _d(dL_dout)
        out = dict(dmean2D=np.empty((P, 4)), dconic=np.empty((P, 4)), dopacity=np.empty(P),
                   dcolor=np.empty((P, 3)), dmean3D=np.empty((P, 3)), dcov3D=np.empty((P, 6)),
                   ddc=np.empty((P, 1, 3)), dsh=np.empty((P, max(M, 0), 3)), dscale=np.empty((P, 3)),
                   drot=np.empty((P, 4)))
        self.lib.orc_backward(self.h, _p(dL), *[_p(out[k]) for k in ("dmean2D", "dconic", "dopacity", "dcolor",
                                                                     "dmean3D", "dcov3D", "ddc", "dsh", "dscale",
                                                                     "drot")])
        return out

    def render_simp(self, eps_alpha=1e-5, eps_T=1e-5, eps_w=1e-5):
        """Importance pass on the current records and lists: per-Gaussian weight sums, counts, max counts."""
        P = self.P
        w, c, m, amb = np.empty(P), np.empty(P, np.int32), np.empty(P), np.empty(P, np.uint8)
        self.lib.orc_render_simp(self.h, float(eps_alpha), float(eps_T), float(eps_w), _p(w), _p(c), _p(m), _p(amb))
        return dict(weights=w, counts=c, max_counts=m, ambiguous=amb.astype(bool))

    def render_depth(self, eps_alpha=1e-5, eps_T=1e-5, eps_w=1e-5):
        """Depth pass on the current records and lists (per-pixel outputs, ambiguity flags)."""
        H, W = self.H, self.W
        pts, d, a, dsc = np.empty((3, H, W)), np.empty((H, W)), np.empty((H, W)), np.empty((H, W))
        g, amb = np.empty((H, W), np.int32), np.empty((H, W), np.uint8)
        self.lib.orc_render_depth(self.h, float(eps_alpha), float(eps_T), float(eps_w), _p(pts), _p(d), _p(a),
                                  _p(g), _p(dsc), _p(amb))
        return dict(out_pts=pts, out_depth=d, accum_alpha=a, gidx=g, discriminants=dsc, ambiguous=amb.astype(bool))

    def densify(self, dmean2D, grad_accum=None, grad_accum_abs=None, max_radii=None, denom=None):
        arrs = [_d(dmean2D), _d(grad_accum), _d(grad_accum_abs), _d(max_radii), _d(denom)]
        self.lib.orc_densify(self.h, *[_p(a) for a in arrs])
        return arrs[1:]


def num_threads() -> int:
    return int(load().orc_num_threads())


def set_threads(n: int) -> None:
    load().orc_set_threads(int(n))


def eval_sh(deg: int, dirs, coeffs):
    """SH colour without offset/clamp; coeffs (n, 16, 3), coefficient 0 = DC."""
    dirs, coeffs = _d(dirs), _d(coeffs)
    out = np.empty((dirs.shape[0], 3))
    load().orc_eval_sh(dirs.shape[0], int(deg), _p(dirs), _p(coeffs), _p(out))
    return out


def cov3d(scales, quats, scale_modifier: float = 1.0):
    """Upper triangle (xx, xy, xz, yy, yz, zz) of R diag(s^2) R^T, raw quaternions."""
    scales, quats = _d(scales), _d(quats)
    out = np.empty((scales.shape[0], 6))
    load().orc_cov3d(scales.shape[0], _p(scales), _p(quats), float(scale_modifier), _p(out))
    return out


def sparse_adam(param, grad, exp_avg, exp_avg_sq, visible, lr: float, step: int, eps: float, b1: float = 0.9,
                b2: float = 0.999):
    """FB's SparseGaussianAdam.step for one parameter group, in FP32 as FB computes it.

    FB __init__.py:288-298: the step count t is advanced first and the kernel is
    given lr sqrt(1 - 0.999^t) / (1 - 0.9^t); adam.cu:26-37: for rows with
    visible[i], m = b1 m + (1 - b1) g, v = b2 v + (1 - b2) g g,
    p += -lr m / (sqrt(v) + eps); other rows are untouched.  Returns new
    (param, exp_avg, exp_avg_sq) arrays of param's shape.
    """
    f = np.float32
    t = f(step)
    lr_t = f(f(lr) * np.sqrt(f(1) - f(0.999) ** t) / (f(1) - f(0.9) ** t))
    N = len(visible)
    p, g = np.asarray(param, f).reshape(N, -1), np.asarray(grad, f).reshape(N, -1)
    m, v = np.asarray(exp_avg, f).reshape(N, -1), np.asarray(exp_avg_sq, f).reshape(N, -1)
    b1, b2, eps = f(b1), f(b2), f(eps)
    m_new = b1 * m + (f(1) - b1) * g
    v_new = b2 * v + (f(1) - b2) * g * g
    p_new = p + (-lr_t) * m_new / (np.sqrt(v_new) + eps)
    vis = np.asarray(visible, bool)[:, None]
    shape = np.shape(param)
    return (np.where(vis, p_new, p).reshape(shape), np.where(vis, m_new, m).reshape(shape),
            np.where(vis, v_new, v).reshape(shape))


def activation_grad(kind: str, raw, grad_out):
    """dL/draw from dL/dactivated for the 3DGS activations (FP64): sigmoid (y' = (1 - y) y),
    exp (y' = y) and normalize along the last axis (dL/dx = g / |x| - x (g . x) / |x|^3)."""
    raw, g = np.asarray(raw, np.float64), np.asarray(grad_out, np.float64)
    if kind == "sigmoid":
        y = 1.0 / (1.0 + np.exp(-raw))
        return g * (1.0 - y) * y
    if kind == "exp":
        return g * np.exp(raw)
    if kind == "normalize":
        n = np.linalg.norm(raw, axis=-1, keepdims=True)
        return g / n - raw * (g * raw).sum(-1, keepdims=True) / n ** 3
    if kind == "identity":
        return g
    raise ValueError(kind)


def ssim_window() -> np.ndarray:
    """11-tap Gaussian of sigma 1.5, normalised (3DGS utils/loss_utils.py:23-25), FP64."""
    t = np.arange(11, dtype=np.float64) - 5.0
    g = np.exp(-t * t / (2.0 * 1.5 * 1.5))
    return g / g.sum()


def _window_sum(a):
    """Separable 11x11 window sum of the last two axes with zero padding ("same"),
    the F.conv2d(..., padding=5) of 3DGS utils/loss_utils.py:44-52."""
    w = ssim_window()
    H, W = a.shape[-2:]
    p = np.zeros(a.shape[:-2] + (H + 10, W + 10))
    p[..., 5:5 + H, 5:5 + W] = a
    h = sum(w[t] * p[..., :, t:t + W] for t in range(11))
    return sum(w[t] * h[..., t:t + H, :] for t in range(11))


def ssim_map(img1, img2, C1: float = 0.01 ** 2, C2: float = 0.03 ** 2):
    """SSIM map and its partials w.r.t. mu1, E[x^2], E[xy] (FP64), as fused-ssim returns them
    (ssim.cu:262-283; the map of 3DGS loss_utils.py:44-60).  Arrays (..., H, W)."""
    x, y = np.asarray(img1, np.float64), np.asarray(img2, np.float64)
    return ssim_from_moments(_window_sum(x), _window_sum(y), _window_sum(x * x), _window_sum(y * y),
                             _window_sum(x * y), C1, C2)


def ssim_from_moments(mu1, mu2, e11, e22, e12, C1: float = 0.01 ** 2, C2: float = 0.03 ** 2):
    """SSIM and its partials w.r.t. mu1, E[x^2], E[xy] from the five window moments (FP64)."""
    s1, s2, s12 = e11 - mu1 * mu1, e22 - mu2 * mu2, e12 - mu1 * mu2
    C = 2 * mu1 * mu2 + C1
    D = 2 * s12 + C2
    A = mu1 * mu1 + mu2 * mu2 + C1
    B = s1 + s2 + C2
    m = C * D / (A * B)
    d_mu1 = (2 * mu2 * D - 2 * mu2 * C) / (A * B) - 2 * mu1 * C * D / (A * A * B) + 2 * mu1 * C * D / (A * B * B)
    return m, d_mu1, -C * D / (A * B * B), 2 * C / (A * B)


def ssim_backward(img1, img2, dL_dmap, d_mu1, d_e11, d_e12):
    """dL/dimg1 = G * (g dm/dmu1) + 2 x G * (g dm/dE[x^2]) + y G * (g dm/dE[xy]) (fused-ssim
    ssim.cu:287-365; the window is symmetric, so its transpose is itself)."""
    g = np.asarray(dL_dmap, np.float64)
    x, y = np.asarray(img1, np.float64), np.asarray(img2, np.float64)
    return _window_sum(g * d_mu1) + 2 * x * _window_sum(g * d_e11) + y * _window_sum(g * d_e12)


def l1_dssim(img, gt, lam: float):
    """The backbones' training loss (1 - lam) mean|img - gt| + lam (1 - mean SSIM) and its
    gradient w.r.t. img (taming-3dgs/train_faster.py:121-125), FP64: (loss, ssim_mean, grad)."""
    x, y = np.asarray(img, np.float64), np.asarray(gt, np.float64)
    n = x.size
    m, a, b, c = ssim_map(x, y)
    grad = (1.0 - lam) * np.sign(x - y) / n + ssim_backward(x, y, np.full_like(m, -lam / n), a, b, c)
    return (1.0 - lam) * np.abs(x - y).mean() + lam * (1.0 - m.mean()), m.mean(), grad
