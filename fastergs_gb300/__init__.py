"""GB300-native differentiable Gaussian rasterizer, a drop-in for FasterGS's
``diff_gaussian_rasterization_faster`` backend.

Same public names and behaviour as FB's
gs_submodules/diff-gaussian-rasterization_faster/diff_gaussian_rasterization_faster/__init__.py:
``GaussianRasterizationSettings``, ``GaussianRasterizer``, ``rasterize_gaussians``,
the ``_RasterizeGaussians`` autograd Function, the persistent ``Buffer`` and
``SparseGaussianAdam``.  Every op runs on hand-written sm_103a kernels behind
the C ABI in include/fgs.h; there is no CPU or PyTorch fallback.

Differences that only show where FB would fail:
  * the key-capacity overflow raises ``RuntimeError("Too many k-v pairs!")``
    (FB raises a bare string, itself a TypeError) and nothing is written past
    the capacity;
  * ``Buffer`` is allocated on first use, not at import, so importing the
    package does not need a GPU;
  * ``cov3D_precomp`` raises NotImplementedError (FB accepts it, ignores it
    and reads the absent scales);
  * a backward whose forward's pair lists were overwritten by a later
    forward (the shared ``Buffer`` holds one frame) raises RuntimeError; FB
    silently differentiates the later frame's lists.
"""
from __future__ import annotations

from typing import NamedTuple

import torch
import torch.nn as nn

from . import _C, _lib

__all__ = ["GaussianRasterizationSettings", "GaussianRasterizer", "rasterize_gaussians", "Buffer",
           "SparseGaussianAdam", "_RasterizeGaussians", "_C", "cpu_deep_copy_tuple"]

_EXT = None


def _ext():
    """The compiled extension (``diff_gaussian_rasterization_faster._C``) the drop-in path runs on.

    Its ``ops`` are ``_C.ops`` compiled: the same C ABI calls without the
    per-call ctypes and Python argument handling.  Missing means unbuilt, and
    that is an error, not a reason to take another path."""
    global _EXT
    if _EXT is None:
        try:
            from diff_gaussian_rasterization_faster import _C as ext
        except ImportError as e:
            raise ImportError("the compiled extension diff_gaussian_rasterization_faster._C is missing: build it "
                              "with fastergs_gb300.build.build()") from e
        _EXT = ext
    return _EXT


def cpu_deep_copy_tuple(input_tuple):
    """Host copies of the tensors of a tuple, other items as they are (FB __init__.py:16-18)."""
    return tuple(item.cpu().clone() if isinstance(item, torch.Tensor) else item for item in input_tuple)


class Buffer:
    """Persistent device buffers shared by all calls (FB __init__.py:21-38)."""

    def __init__(self, device="cuda", MAX_NUM_RENDERED=2**24, MAX_NUM_TILES=2**20, **kwargs):
        i64, i32 = torch.int64, torch.int32
        self.gaussian_keys_unsorted = torch.zeros(MAX_NUM_RENDERED, device=device, dtype=i64)
        self.gaussian_values_unsorted = torch.zeros(MAX_NUM_RENDERED, device=device, dtype=i32)
        self.gaussian_keys_sorted = torch.zeros(MAX_NUM_RENDERED, device=device, dtype=i64)
        self.gaussian_values_sorted = torch.zeros(MAX_NUM_RENDERED, device=device, dtype=i32)
        self.MAX_NUM_RENDERED = MAX_NUM_RENDERED
        self.MAX_NUM_TILES = MAX_NUM_TILES
        self.SORT_BUFFER_SIZE = _C.ops.get_sort_buffer_size(MAX_NUM_RENDERED)
        self.list_sorting_space = torch.zeros(self.SORT_BUFFER_SIZE, device=device, dtype=torch.int8)
        self.ranges = torch.zeros((MAX_NUM_TILES, 2), device=device, dtype=i32)
        self.curr_offset = torch.zeros(1, device=device, dtype=i32)
        self.splat_buffer = torch.zeros([MAX_NUM_RENDERED, 32], device=device, dtype=torch.float32)
        self.device = device
        # frames binned into this buffer so far; a backward checks that its
        # forward's frame is still the one the buffer holds
        self.generation = 0


_HOST_COUNTS: dict = {}


def _host_counts(dev) -> torch.Tensor:
    """Pinned host words the forward reads the pair and task counts into."""
    key = (dev.type, dev.index)
    if key not in _HOST_COUNTS:
        _HOST_COUNTS[key] = torch.zeros(2, dtype=torch.int32).pin_memory()
    return _HOST_COUNTS[key]


def _bin(buffer, rs, means3D, dc, shs, colors_precomp, opacities, scales, rotations, culling):
    """Preprocess and sort into the shared Buffer (FB __init__.py:96-119): returns (radii, num_rendered)."""
    buffer.generation = getattr(buffer, "generation", 0) + 1
    ext = _ext()
    buffer.curr_offset.fill_(0)
    radii = ext.ops.preprocess(
        rs.sh_degree, means3D, colors_precomp, dc, shs, opacities, scales, rotations, rs.scale_modifier,
        rs.image_width, rs.image_height, 16, 16, rs.campos, rs.viewmatrix, rs.projmatrix, rs.tanfovx, rs.tanfovy,
        100.0, 0.01, buffer.gaussian_keys_unsorted, buffer.gaussian_values_unsorted, buffer.gaussian_values_sorted,
        buffer.curr_offset, rs.mult, buffer.splat_buffer, culling)
    # One host read per frame (FB's K read): the pair count and the
    # large-footprint task count, stored into pinned memory by a kernel (no
    # copy-engine queueing behind the caller's own transfers), one
    # synchronisation, and the sort (FB's sort_gaussian) launched from the same
    # C++ call when the pairs fit, so the GPU waits on no Python in between.
    counts = _host_counts(means3D.device)
    num_rendered, num_tasks = ext.count_and_sort(
        buffer.curr_offset, counts, buffer.MAX_NUM_RENDERED, buffer.gaussian_values_sorted.numel(), rs.image_width,
        rs.image_height, 16, 16, buffer.list_sorting_space, buffer.gaussian_keys_unsorted,
        buffer.gaussian_values_unsorted, buffer.gaussian_keys_sorted, buffer.gaussian_values_sorted)
    if num_rendered >= buffer.MAX_NUM_RENDERED or num_tasks > buffer.gaussian_values_sorted.numel() // 2:
        _C.device_errors(means3D.device)  # clears the capacity bit the skipped writes latched
        if num_rendered >= buffer.MAX_NUM_RENDERED:
            raise RuntimeError("Too many k-v pairs!")
        raise RuntimeError("preprocess overflowed a device queue (too many large Gaussians)")
    return radii, num_rendered


class _LazyBuffer:
    """Class attribute that allocates the shared Buffer on first access."""

    def __init__(self):
        self._buf = None

    def __get__(self, obj, owner):
        if self._buf is None:
            self._buf = Buffer()
        return self._buf

    def __set__(self, obj, value):  # pragma: no cover - instances never set it
        self._buf = value


def rasterize_gaussians(means3D, dc, shs, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                        raster_settings, culling, xyz_gradient_accum, xyz_gradient_accum_abs, max_radii, denom,
                        adam=None):
    return _RasterizeGaussians.apply(means3D, dc, shs, colors_precomp, opacities, scales, rotations,
                                     cov3Ds_precomp, raster_settings, culling, xyz_gradient_accum,
                                     xyz_gradient_accum_abs, max_radii, denom, adam)


class _RasterizeGaussians(torch.autograd.Function):
    """FB __init__.py:76-187: preprocess -> sort -> render_16x16, backward through _C.ops.backward."""

    buffer = _LazyBuffer()

    @staticmethod
    def forward(ctx, means3D, dc, shs, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                raster_settings, culling, xyz_gradient_accum, xyz_gradient_accum_abs, max_radii, denom, adam=None):
        if adam is not None:
            adam._check_fused(means3D, dc, shs, colors_precomp)
        buffer = _RasterizeGaussians.buffer
        splat_buffer = buffer.splat_buffer
        N = means3D.shape[0]
        radii, num_rendered = _bin(buffer, raster_settings, means3D, dc, shs, colors_precomp, opacities, scales,
                                   rotations, culling)
        H, W = raster_settings.image_height, raster_settings.image_width
        # every pixel is written by the merge, so no zero-fill is needed
        last_contributor = torch.empty((H, W, 1), device=means3D.device, dtype=torch.int)
        Ts_final = torch.empty((H, W, 1), device=means3D.device, dtype=torch.float)
        bucket_sum, out_color, img_buffer, smp_buffer = _ext().ops.render_16x16(
            N, num_rendered, W, H, splat_buffer, buffer.gaussian_keys_sorted, buffer.gaussian_values_sorted,
            buffer.ranges, raster_settings.bg, last_contributor, Ts_final, read_bucket_sum=False)
        ctx.raster_settings = raster_settings
        ctx.adam = adam
        ctx.num_rendered = num_rendered
        ctx.buffer = buffer
        ctx.generation = buffer.generation
        ctx.bucket_sum = bucket_sum
        ctx.save_for_backward(means3D, scales, rotations, dc, shs, opacities, out_color, last_contributor,
                              Ts_final, radii, splat_buffer, img_buffer, smp_buffer, xyz_gradient_accum,
                              xyz_gradient_accum_abs, max_radii, denom)
        return out_color, radii

    @staticmethod
    def backward(ctx, grad_out_color, _):
        rs = ctx.raster_settings
        buffer = ctx.buffer
        if getattr(buffer, "generation", 0) != ctx.generation:
            raise RuntimeError("the rasterizer's shared Buffer holds a later frame than this backward's forward: "
                               "call backward before the next forward (or render_simp / render_depth)")
        zFar, zNear = 100.0, 0.01
        (means3D, scales, rotations, dc, shs, opacities, out_color, last_contributor, Ts_final, radii,
         splat_buffer, img_buffer, smp_buffer, xyz_gradient_accum, xyz_gradient_accum_abs, max_radii,
         denom) = ctx.saved_tensors
        if ctx.adam is not None:
            # sparse Adam fused into the backward: the raw parameters are stepped
            # in place and autograd receives no gradient for them
            fused, _keep, _ = ctx.adam._fused_args(means3D.shape[0], means3D.device)
            _C.backward_adam(
                rs.sh_degree, ctx.bucket_sum, means3D, radii, shs, opacities, scales, rotations, rs.scale_modifier,
                rs.image_width, rs.image_height, 16, 16, rs.tanfovx, rs.tanfovy, rs.campos, rs.viewmatrix,
                rs.projmatrix, img_buffer, smp_buffer, splat_buffer, buffer.gaussian_values_sorted, buffer.ranges,
                rs.bg, last_contributor, Ts_final, grad_out_color.contiguous(), fused, xyz_gradient_accum,
                xyz_gradient_accum_abs, max_radii, denom)
            return (None,) * 15
        (grad_mean2D, grad_color, grad_opacity, grad_mean3D, grad_cov3D, grad_dc, grad_shs, grad_scales,
         grad_rotations) = _ext().ops.backward(
            rs.sh_degree, ctx.bucket_sum, means3D, radii, dc, shs, opacities, scales, rotations,
            rs.scale_modifier, rs.image_width, rs.image_height, 16, 16, rs.tanfovx, rs.tanfovy, zFar, zNear,
            rs.campos, rs.viewmatrix, rs.projmatrix, img_buffer, smp_buffer, splat_buffer,
            buffer.gaussian_values_sorted, buffer.ranges, rs.bg, last_contributor, Ts_final,
            grad_out_color.contiguous(), xyz_gradient_accum, xyz_gradient_accum_abs, max_radii, denom,
            abs_grad=_C._nonempty(xyz_gradient_accum_abs),  # dmean2D is not returned to autograd
            minimal=True)
        grad_color = grad_color if grad_color.numel() else None      # only precomputed colours need it
        grad_cov3D = None                                             # covariances are never precomputed here
        return (grad_mean3D, grad_dc, grad_shs, grad_color, grad_opacity, grad_scales, grad_rotations, grad_cov3D,
                None, None, None, None, None, None, None)


class GaussianRasterizationSettings(NamedTuple):
    """FB __init__.py:191-204."""
    image_height: int
    image_width: int
    tanfovx: float
    tanfovy: float
    bg: torch.Tensor
    scale_modifier: float
    viewmatrix: torch.Tensor
    projmatrix: torch.Tensor
    sh_degree: int
    campos: torch.Tensor
    mult: float
    prefiltered: bool
    debug: bool


class GaussianRasterizer(nn.Module):
    """FB __init__.py:207-264."""

    def __init__(self, raster_settings, **kwargs):
        super().__init__()
        self.raster_settings = raster_settings

    def forward(self, means3D, opacities, dc=None, shs=None, colors_precomp=None, scales=None, rotations=None,
                cov3D_precomp=None, culling=None, xyz_gradient_accum=None, xyz_gradient_accum_abs=None,
                max_radii=None, denom=None, adam=None):
        """FB's arguments, plus ``adam``: a SparseGaussianAdam whose step is fused into this frame's
        backward (the raw parameters are stepped during ``loss.backward()``; do not call its
        ``step`` for the frame).  Only the image loss reaches the parameters in that mode."""
        if (shs is None and colors_precomp is None) or (shs is not None and colors_precomp is not None):
            raise Exception('Please provide excatly one of either SHs or precomputed colors!')
        if ((scales is None or rotations is None) and cov3D_precomp is None) or \
                ((scales is not None or rotations is not None) and cov3D_precomp is not None):
            raise Exception('Please provide exactly one of either scale/rotation pair or precomputed 3D covariance!')
        empty = torch.tensor([])
        dc = empty if dc is None else dc
        shs = empty if shs is None else shs
        culling = torch.tensor([], dtype=torch.bool) if culling is None else culling
        colors_precomp = empty if colors_precomp is None else colors_precomp
        scales = empty if scales is None else scales
        rotations = empty if rotations is None else rotations
        cov3D_precomp = empty if cov3D_precomp is None else cov3D_precomp
        xyz_gradient_accum = empty if xyz_gradient_accum is None else xyz_gradient_accum
        xyz_gradient_accum_abs = empty if xyz_gradient_accum_abs is None else xyz_gradient_accum_abs
        max_radii = empty if max_radii is None else max_radii
        denom = empty if denom is None else denom
        return rasterize_gaussians(means3D, dc, shs, colors_precomp, opacities, scales, rotations, cov3D_precomp,
                                   self.raster_settings, culling, xyz_gradient_accum, xyz_gradient_accum_abs,
                                   max_radii, denom, adam)


def _inputs(means3D, opacities, dc, shs, colors_precomp, scales, rotations, culling):
    empty = torch.tensor([])
    return (empty if dc is None else dc, empty if shs is None else shs,
            empty if colors_precomp is None else colors_precomp,
            empty if scales is None else scales, empty if rotations is None else rotations,
            torch.tensor([], dtype=torch.bool) if culling is None else culling)


def _render_simp(self, means3D, opacities, dc=None, shs=None, colors_precomp=None, scales=None, rotations=None,
                 cov3D_precomp=None, culling=None):
    """Importance pass (FB _C.ops.render_simp, called as Mini-Splatting 2's faster renderer does,
    mini-splatting2/gaussian_renderer/render_faster.py:181): returns (radii, accum_weights (P,),
    accum_weights_count (P,), accum_max_count (P,))."""
    if cov3D_precomp is not None:
        raise NotImplementedError("precomputed 3D covariances are not supported (FB needs scales and rotations)")
    dc, shs, colors_precomp, scales, rotations, culling = _inputs(means3D, opacities, dc, shs, colors_precomp,
                                                                  scales, rotations, culling)
    rs = self.raster_settings
    buffer = _RasterizeGaussians.buffer
    with torch.no_grad():
        radii, K = _bin(buffer, rs, means3D, dc, shs, colors_precomp, opacities, scales, rotations, culling)
        _, w, cnt, mx = _ext().ops.render_simp(means3D.shape[0], K, rs.image_width, rs.image_height,
                                               buffer.splat_buffer, buffer.gaussian_keys_sorted,
                                               buffer.gaussian_values_sorted, buffer.ranges)
    return radii, w, cnt, mx


def _render_depth(self, means3D, opacities, dc=None, shs=None, colors_precomp=None, scales=None, rotations=None,
                  cov3D_precomp=None, culling=None):
    """Depth pass (FB _C.ops.render_depth, called as Mini-Splatting 2's faster renderer does,
    mini-splatting2/gaussian_renderer/render_faster.py:238): returns a dict with "out_pts" (3,H,W),
    "rendered_depth", "accum_alpha", "gidx", "discriminants" (1,H,W) and "radii"."""
    if cov3D_precomp is not None:
        raise NotImplementedError("precomputed 3D covariances are not supported (FB needs scales and rotations)")
    dc, shs, colors_precomp, scales, rotations, culling = _inputs(means3D, opacities, dc, shs, colors_precomp,
                                                                  scales, rotations, culling)
    rs = self.raster_settings
    buffer = _RasterizeGaussians.buffer
    with torch.no_grad():
        radii, K = _bin(buffer, rs, means3D, dc, shs, colors_precomp, opacities, scales, rotations, culling)
        pts, depth, alpha, gidx, disc = _ext().ops.render_depth(
            means3D.shape[0], K, rs.image_width, rs.image_height, buffer.splat_buffer, buffer.gaussian_keys_sorted,
            buffer.gaussian_values_sorted, buffer.ranges, means3D, scales, rotations, rs.projmatrix, rs.campos)
    return {"out_pts": pts, "rendered_depth": depth, "discriminants": disc, "gidx": gidx, "accum_alpha": alpha,
            "radii": radii}


GaussianRasterizer.render_simp = _render_simp
GaussianRasterizer.render_depth = _render_depth


class SparseGaussianAdam(torch.optim.Adam):
    """Adam that only steps the rows of visible Gaussians (FB __init__.py:267-298).

    ``step(visibility, N)`` is FB's.  Passed as ``adam=`` to the rasterizer, the
    same step runs inside the frame's backward instead: the gradients of the
    six named groups (xyz, f_dc, f_rest, opacity, scaling, rotation, as
    FasterGS's backbones name them) never reach memory; the activations
    opacity = sigmoid, scaling = exp, rotation = normalize are differentiated
    in the kernel (``activations`` overrides them with "identity").
    """

    _DEFAULT_ACTS = {"opacity": "sigmoid", "scaling": "exp", "rotation": "normalize"}
    _WIDTH = {"xyz": 3, "f_dc": 3, "opacity": 1, "scaling": 3, "rotation": 4}

    def __init__(self, params, lr, eps, activations=None):
        super().__init__(params=params, lr=lr, eps=eps)
        self.activations = dict(self._DEFAULT_ACTS, **(activations or {}))

    def _named(self):
        named = {}
        for group in self.param_groups:
            name = group.get("name")
            if name in _lib.ADAM_GROUPS:
                if len(group["params"]) != 1:
                    raise ValueError(f"group {name!r} must hold exactly one tensor")
                named[name] = group
        return named

    def _check_fused(self, means3D, dc, shs, colors_precomp):
        """The fused step applies the rasterizer's gradients to the raw tensors: xyz, f_dc and f_rest
        must be the tensors passed as means3D, dc and shs."""
        if colors_precomp is not None and colors_precomp.numel():
            raise ValueError("the fused Adam step needs SH colours (no precomputed colours)")
        named = self._named()
        if not named:
            raise ValueError("no parameter group is named xyz, f_dc, f_rest, opacity, scaling or rotation")
        for name, t in (("xyz", means3D), ("f_dc", dc), ("f_rest", shs)):
            if name in named and (t is None or named[name]["params"][0].data_ptr() != t.data_ptr()):
                raise ValueError(f"group {name!r} must be the tensor passed to the rasterizer")

    @torch.no_grad()
    def _fused_args(self, N, device, advance: bool = True, lr_device: torch.Tensor | None = None):
        """One fused step's fgs_adam_fused: initialises the state lazily, advances each group's step
        (unless advance=False) and sets FB's bias-compensated step sizes
        (lr sqrt(1 - 0.999^t) / (1 - 0.9^t)) by value, or points the kernel at lr_device (6 device
        floats the caller fills).  Returns (struct, tensors to keep alive, step sizes on the host)."""
        fused = _lib.AdamFused()
        lrs = torch.zeros(len(_lib.ADAM_GROUPS), dtype=torch.float32)
        keep = []
        named = self._named()
        for gi, name in enumerate(_lib.ADAM_GROUPS):
            group = named.get(name)
            if group is None:
                continue
            param = group["params"][0]
            if param.numel() == 0:
                continue
            width = self._WIDTH.get(name)
            if (width is not None and param.numel() != N * width) or param.numel() % max(N, 1):
                raise ValueError(f"group {name!r} does not hold {N} Gaussians")
            if not (param.is_contiguous() and param.dtype == torch.float32 and param.device == device):
                raise TypeError(f"group {name!r} must be a contiguous float32 tensor on {device}")
            state = self.state[param]
            if len(state) == 0:
                state['step'] = torch.tensor(0.0, dtype=torch.float32)
                state['exp_avg'] = torch.zeros_like(param, memory_format=torch.preserve_format)
                state['exp_avg_sq'] = torch.zeros_like(param, memory_format=torch.preserve_format)
            if advance:
                state['step'] += 1
            step = state['step']
            if step > 0:
                lrs[gi] = group["lr"] * (1 - 0.999 ** step) ** 0.5 / (1 - 0.9 ** step)
            fused.param[gi] = param.data_ptr()
            fused.exp_avg[gi] = state['exp_avg'].data_ptr()
            fused.exp_avg_sq[gi] = state['exp_avg_sq'].data_ptr()
            fused.eps[gi] = float(group["eps"])
            keep.append(param)
        for gi in range(len(_lib.ADAM_GROUPS)):
            fused.lr_value[gi] = float(lrs[gi])
        fused.lr = lr_device.data_ptr() if lr_device is not None else None
        fused.b1, fused.b2 = 0.9, 0.999
        acts = self.activations
        fused.opacity_act = _lib.ACT[acts["opacity"]]
        fused.scaling_act = _lib.ACT[acts["scaling"]]
        fused.rotation_act = _lib.ACT[acts["rotation"]]
        return fused, keep, lrs

    @torch.no_grad()
    def step(self, visibility, N):
        for group in self.param_groups:
            lr = group["lr"]
            eps = group["eps"]
            assert len(group["params"]) == 1, "more than one tensor in group"
            param = group["params"][0]
            if param.grad is None or param.grad.numel() == 0:
                continue
            state = self.state[param]
            if len(state) == 0:
                state['step'] = torch.tensor(0.0, dtype=torch.float32)
                state['exp_avg'] = torch.zeros_like(param, memory_format=torch.preserve_format)
                state['exp_avg_sq'] = torch.zeros_like(param, memory_format=torch.preserve_format)
            exp_avg = state["exp_avg"]
            exp_avg_sq = state["exp_avg_sq"]
            state['step'] += 1
            step = state['step']
            M = param.numel() // N
            _ext().ops.adamUpdate(param, param.grad, exp_avg, exp_avg_sq, visibility,
                                  float(lr * (1 - 0.999 ** step) ** 0.5 / (1 - 0.9 ** step)), 0.9, 0.999, eps, N, M)
