"""``_C`` of the rasterizer: the ``ops`` namespace FB's Python layer calls.

Mirrors FB csrc/pybind.cpp:135-416 (``_C.ops.preprocess``, ``sort_gaussian``,
``get_sort_buffer_size``, ``render_16x16``, ``backward``, ``adamUpdate``,
``render_simp``, ``render_depth``) with the same argument order, tensor
shapes and dtypes.  Each op validates its tensors, takes raw device pointers
and calls the C ABI of libfgs.so on torch's current stream.  Outputs are
allocated with torch, as in FB.

Also exports ``rasterize_gaussians`` / ``rasterize_gaussians_backward`` with
the signature of the vanilla 3DGS extension
(gs_submodules/diff-gaussian-rasterization/rasterize_points.h:18-59) over the
same C ABI.
"""
from __future__ import annotations

import ctypes as C
from types import SimpleNamespace

import torch

from . import _lib

TILE = 16
BUCKET = 128
# Sample-state rows are sized so the buffer's first dimension encodes the
# bucket capacity the forward reserved: rows = max_buckets + 1.
_SAMPLE_ROW = 4120  # per bucket: 256 x 16-byte samples, owner tile, queue slot, live-list entry


def _ptr(t: torch.Tensor | None) -> int:
    if t is None or t.numel() == 0:
        return 0
    return t.data_ptr()


def _stream(dev: torch.device) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


def _f32(name: str, t: torch.Tensor, dev: torch.device) -> torch.Tensor:
    """Contiguous float32 tensor on dev, or an empty tensor for 'absent'."""
    if t is None or t.numel() == 0:
        return torch.empty(0)
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    if t.device != dev:
        raise ValueError(f"{name} must be on {dev}, got {t.device}")
    return t.contiguous()


_COUNTERS: dict = {}


def _counters(dev: torch.device) -> torch.Tensor:
    """The preprocess's work counters (zeroed and then counted into by every
    call), one set per (device, stream): calls in flight on different
    streams of one device each count into their own."""
    key = (dev.type, dev.index, _stream(dev))
    if key not in _COUNTERS:
        _COUNTERS[key] = torch.zeros(16, dtype=torch.int32, device=dev)
    return _COUNTERS[key]


def _nonempty(t) -> bool:
    return t is not None and t.numel() != 0


def _device_of(t: torch.Tensor) -> torch.device:
    if not t.is_cuda:
        raise ValueError("the rasterizer runs on CUDA tensors only (no CPU fallback)")
    return t.device


def preprocess(deg, orig_points, color_precomp, dc, shs, opacities, scales, rotations, scale_modifier,
               width, height, block_x, block_y, campos, view_matrix, proj_matrix, tan_fovx, tan_fovy,
               zFar, zNear, gaussian_keys_unsorted, gaussian_values_unsorted, gaussian_values_sorted,
               curr_offset, mult, splat_buffer, culling):
    """FB pybind.cpp:26-76.  Returns radii (P,) int32; appends pairs at curr_offset."""
    dev = _device_of(opacities)
    P = opacities.size(0)
    M = shs.size(1) if shs.numel() and shs.size(0) != 0 else 0
    means = _f32("means3D", orig_points, dev)
    colors = _f32("colors_precomp", color_precomp, dev)
    dcc = _f32("dc", dc, dev)
    shc = _f32("shs", shs, dev)
    op = _f32("opacities", opacities, dev)
    sc = _f32("scales", scales, dev)
    ro = _f32("rotations", rotations, dev)
    if sc.numel() == 0 or ro.numel() == 0:
        raise NotImplementedError("precomputed 3D covariances are not supported: FB ignores cov3D_precomp and "
                                  "needs scales and rotations (FB __init__.py:107-115)")
    cam = _f32("campos", campos, dev)
    vm = _f32("viewmatrix", view_matrix, dev)
    pm = _f32("projmatrix", proj_matrix, dev)
    cull = culling.to(dev).contiguous() if culling is not None and culling.numel() else None
    if cull is not None and cull.dtype != torch.bool:
        raise TypeError("culling must be a bool tensor")
    for name, t, dt in (("gaussian_keys_unsorted", gaussian_keys_unsorted, torch.int64),
                        ("gaussian_values_unsorted", gaussian_values_unsorted, torch.int32),
                        ("gaussian_values_sorted", gaussian_values_sorted, torch.int32),
                        ("curr_offset", curr_offset, torch.int32), ("splat_buffer", splat_buffer, torch.float32)):
        if t.dtype != dt or not t.is_contiguous() or t.device != dev:
            raise TypeError(f"{name} must be a contiguous {dt} tensor on {dev}")
    radii = torch.empty(P, dtype=torch.int32, device=dev)
    cap = min(gaussian_keys_unsorted.numel(), gaussian_values_unsorted.numel())
    _lib.call("fgs_preprocess", int(P), int(deg), int(M), _ptr(means), _ptr(colors), _ptr(dcc), _ptr(shc),
              _ptr(op), _ptr(sc), _ptr(ro), float(scale_modifier), int(width), int(height), int(block_x),
              int(block_y), _ptr(cam), _ptr(vm), _ptr(pm), float(tan_fovx), float(tan_fovy), float(zFar),
              float(zNear), float(mult), _ptr(cull), _ptr(splat_buffer), int(splat_buffer.size(0)),
              _ptr(gaussian_keys_unsorted), _ptr(gaussian_values_unsorted), int(cap),
              _ptr(gaussian_values_sorted), int(gaussian_values_sorted.numel()), _ptr(curr_offset),
              _ptr(_counters(dev)), _ptr(radii), _stream(dev))
    return radii


def get_sort_buffer_size(num_rendered):
    """FB pybind.cpp:95-98."""
    return int(_lib.load().fgs_sort_temp_bytes(int(num_rendered)))


def sort_gaussian(num_rendered, width, height, block_x, block_y, list_sorting_space, gaussian_keys_unsorted,
                  gaussian_values_unsorted, gaussian_keys_sorted, gaussian_values_sorted):
    """FB pybind.cpp:78-93.  Stable sort of the first num_rendered pairs."""
    dev = _device_of(gaussian_keys_unsorted)
    _lib.call("fgs_sort", int(num_rendered), int(width), int(height), int(block_x), int(block_y),
              _ptr(list_sorting_space), int(list_sorting_space.numel() * list_sorting_space.element_size()),
              _ptr(gaussian_keys_unsorted), _ptr(gaussian_values_unsorted), _ptr(gaussian_keys_sorted),
              _ptr(gaussian_values_sorted), _stream(dev))


def state_sizes(num_rendered, width, height, block_x=TILE, block_y=TILE, bucket_size=BUCKET):
    lib = _lib.load()
    mb = int(lib.fgs_max_buckets(int(num_rendered), int(width), int(height), int(block_x), int(block_y),
                                 int(bucket_size)))
    ib, sb = C.c_size_t(0), C.c_size_t(0)
    _lib.call("fgs_state_bytes", int(width), int(height), int(block_x), int(block_y), mb, C.byref(ib), C.byref(sb))
    return mb, int(ib.value), int(sb.value)


def render_16x16(P, num_rendered, width, height, splat_buffer, gaussian_keys_sorted, gaussian_values_sorted,
                 ranges, bg_color, last_contributor, Ts_final, bucket_size=BUCKET, read_bucket_sum=True):
    """FB pybind.cpp:100-133.  Returns (bucket_sum, out_color (3,H,W), img_buffer, smp_buffer).

    read_bucket_sum=False skips FB's host read of the bucket count (and its
    stream synchronisation) and returns the capacity the sample state was
    sized for instead; this package's backward does not need the count."""
    dev = _device_of(splat_buffer)
    bg = _f32("bg", bg_color, dev)
    if bg.numel() != 3:
        raise ValueError("bg must hold 3 values")
    mb, ib, sb = state_sizes(num_rendered, width, height, TILE, TILE, bucket_size)
    mb = max(mb, 1)
    rows = mb + 1
    if rows * _SAMPLE_ROW < sb:
        raise RuntimeError("sample-state row sizing is inconsistent with the library")
    out_color = torch.empty((3, height, width), dtype=torch.float32, device=dev)
    img_buffer = torch.empty(ib, dtype=torch.uint8, device=dev)
    smp_buffer = torch.empty((rows, _SAMPLE_ROW), dtype=torch.uint8, device=dev)
    bsum = C.c_uint32(0)
    if last_contributor.dtype != torch.int32 or Ts_final.dtype != torch.float32:
        raise TypeError("last_contributor must be int32 and Ts_final float32")
    _lib.call("fgs_render_fwd", int(P), int(num_rendered), int(width), int(height), TILE, TILE, int(bucket_size),
              _ptr(splat_buffer), _ptr(gaussian_keys_sorted), _ptr(gaussian_values_sorted), _ptr(ranges),
              _ptr(bg), _ptr(out_color), _ptr(last_contributor), _ptr(Ts_final), _ptr(img_buffer), ib,
              _ptr(smp_buffer), rows * _SAMPLE_ROW, mb, C.byref(bsum) if read_bucket_sum else None, _stream(dev))
    return (int(bsum.value) if read_bucket_sum else mb), out_color, img_buffer, smp_buffer


def backward(degree, bucket_sum, means3D, radii, dc, sh, opacities, scales, rotations, scale_modifier, width,
             height, block_x, block_y, tan_fovx, tan_fovy, zFar, zNear, campos, viewmatrix, projmatrix, img_func,
             smp_func, splat_buffer, point_list, ranges, background, last_contributor, Ts_final, dL_dout_color,
             xyz_gradient_accum, xyz_gradient_accum_abs, max_radii, denom, bucket_size=BUCKET, abs_grad=True,
             minimal=False):
    """FB pybind.cpp:210-339.  Returns (dL_dmean2D, dL_dcolor, dL_dopacity, dL_dmean3D, dL_dcov3D, dL_ddc,
    dL_dsh, dL_dscale, dL_drot).  abs_grad=False leaves dL_dmean2D[:, 2:] (the |dL/dmean2D| sums,
    read only by the xyz_gradient_accum_abs statistic) at zero and skips their work.  minimal=True
    (the autograd step) returns empty dL_dmean2D and dL_dcov3D, and an empty dL_dcolor when SH
    coefficients are given, without writing them."""
    dev = _device_of(means3D)
    P = means3D.size(0)
    M = sh.size(1) if sh.numel() and sh.size(0) != 0 else 0
    f = dict(dtype=torch.float32, device=dev)
    none = torch.empty(0, **f)
    dmean2D = none if minimal else torch.empty((P, 4), **f)
    dcolor = none if (minimal and sh.numel()) else torch.empty((P, 3), **f)
    dopac = torch.empty((P, 1), **f)
    dmean3D = torch.empty((P, 3), **f)
    dcov3D = none if minimal else torch.empty((P, 6), **f)
    ddc = torch.empty((P, 1, 3), **f)
    dsh = torch.empty((P, M, 3), **f)
    dscale = torch.empty((P, 3), **f)
    drot = torch.empty((P, 4), **f)
    if P == 0:
        return dmean2D, dcolor, dopac, dmean3D, dcov3D, ddc, dsh, dscale, drot
    dconic = none if minimal else torch.empty((P, 2, 2), **f)
    grad_record = torch.empty((P, 12), **f)
    means = _f32("means3D", means3D, dev)
    dcc = _f32("dc", dc, dev)
    shc = _f32("sh", sh, dev)
    sc = _f32("scales", scales, dev)
    ro = _f32("rotations", rotations, dev)
    dL = _f32("dL_dout_color", dL_dout_color, dev)
    bg = _f32("background", background, dev)
    campos = _f32("campos", campos, dev)
    viewmatrix = _f32("viewmatrix", viewmatrix, dev)
    projmatrix = _f32("projmatrix", projmatrix, dev)
    if dL.numel() != 3 * int(width) * int(height):
        raise ValueError("dL_dout_color must be (3, H, W)")
    mb = smp_func.size(0) - 1
    s = _stream(dev)
    _lib.call("fgs_render_bwd", int(P), int(width), int(height), int(block_x), int(block_y), int(bucket_size),
              _ptr(point_list), _ptr(ranges), _ptr(bg), _ptr(splat_buffer), _ptr(Ts_final), _ptr(last_contributor),
              _ptr(img_func), _ptr(smp_func), int(mb), _ptr(dL), _ptr(grad_record), 0 if abs_grad else 1, s)
    stats = xyz_gradient_accum is not None and xyz_gradient_accum.numel() != 0 and xyz_gradient_accum.size(0) != 0
    _lib.call("fgs_preprocess_bwd", int(P), int(degree), int(M), _ptr(means), _ptr(radii), _ptr(dcc), _ptr(shc),
              _ptr(splat_buffer), _ptr(sc), _ptr(ro), float(scale_modifier), _ptr(viewmatrix), _ptr(projmatrix),
              int(width), int(height), float(tan_fovx), float(tan_fovy), _ptr(campos), _ptr(grad_record),
              _ptr(dmean2D), _ptr(dconic), _ptr(dopac), _ptr(dcolor), _ptr(dmean3D), _ptr(dcov3D), _ptr(ddc),
              _ptr(dsh), _ptr(dscale), _ptr(drot),
              _ptr(xyz_gradient_accum) if stats else 0, _ptr(xyz_gradient_accum_abs) if stats else 0,
              _ptr(max_radii) if stats else 0, _ptr(denom) if stats else 0, s)
    return dmean2D, dcolor, dopac, dmean3D, dcov3D, ddc, dsh, dscale, drot


def backward_adam(degree, bucket_sum, means3D, radii, sh, opacities, scales, rotations, scale_modifier, width,
                  height, block_x, block_y, tan_fovx, tan_fovy, campos, viewmatrix, projmatrix, img_func, smp_func,
                  splat_buffer, point_list, ranges, background, last_contributor, Ts_final, dL_dout_color, adam,
                  xyz_gradient_accum, xyz_gradient_accum_abs, max_radii, denom, bucket_size=BUCKET):
    """``backward`` with the sparse Adam step fused into the preprocess backward: the raw parameters
    and moments described by ``adam`` (an ``_lib.AdamFused``) are stepped in place and no gradient
    tensor is produced (FB's step = backward + SparseGaussianAdam.step, __init__.py:267-298)."""
    dev = _device_of(means3D)
    P = means3D.size(0)
    if P == 0:
        return
    M = sh.size(1) if sh.numel() and sh.size(0) != 0 else 0
    grad_record = torch.empty((P, 12), dtype=torch.float32, device=dev)
    means = _f32("means3D", means3D, dev)
    shc = _f32("sh", sh, dev)
    op = _f32("opacities", opacities, dev)
    sc = _f32("scales", scales, dev)
    ro = _f32("rotations", rotations, dev)
    dL = _f32("dL_dout_color", dL_dout_color, dev)
    bg = _f32("background", background, dev)
    campos = _f32("campos", campos, dev)
    viewmatrix = _f32("viewmatrix", viewmatrix, dev)
    projmatrix = _f32("projmatrix", projmatrix, dev)
    if dL.numel() != 3 * int(width) * int(height):
        raise ValueError("dL_dout_color must be (3, H, W)")
    mb = smp_func.size(0) - 1
    s = _stream(dev)
    _lib.call("fgs_render_bwd", int(P), int(width), int(height), int(block_x), int(block_y), int(bucket_size),
              _ptr(point_list), _ptr(ranges), _ptr(bg), _ptr(splat_buffer), _ptr(Ts_final), _ptr(last_contributor),
              _ptr(img_func), _ptr(smp_func), int(mb), _ptr(dL), _ptr(grad_record),
              0 if _nonempty(xyz_gradient_accum_abs) else 1, s)
    stats = xyz_gradient_accum is not None and xyz_gradient_accum.numel() != 0 and xyz_gradient_accum.size(0) != 0
    _lib.call("fgs_preprocess_bwd_adam", int(P), int(degree), int(M), _ptr(means), _ptr(radii), _ptr(shc),
              _ptr(splat_buffer), _ptr(op), _ptr(sc), _ptr(ro), float(scale_modifier), _ptr(viewmatrix),
              _ptr(projmatrix), int(width), int(height), float(tan_fovx), float(tan_fovy), _ptr(campos),
              _ptr(grad_record), C.byref(adam),
              _ptr(xyz_gradient_accum) if stats else 0, _ptr(xyz_gradient_accum_abs) if stats else 0,
              _ptr(max_radii) if stats else 0, _ptr(denom) if stats else 0, s)


def adamUpdate(param, param_grad, exp_avg, exp_avg_sq, visible, lr, b1, b2, eps, N, M):
    """FB pybind.cpp:341-366 (masked Adam over N rows of M values)."""
    dev = _device_of(param)
    for name, t in (("param", param), ("param_grad", param_grad), ("exp_avg", exp_avg),
                    ("exp_avg_sq", exp_avg_sq)):
        if not t.is_contiguous() or t.dtype != torch.float32:
            raise TypeError(f"{name} must be a contiguous float32 tensor")
    vis = visible.contiguous()
    if vis.dtype != torch.bool:
        raise TypeError("visible must be a bool tensor")
    _lib.call("fgs_adam_update", _ptr(param), _ptr(param_grad), _ptr(exp_avg), _ptr(exp_avg_sq), _ptr(vis),
              float(lr), float(b1), float(b2), float(eps), int(N), int(M), _stream(dev))


def render_simp(P, num_rendered, width, height, splat_buffer, gaussian_keys_sorted, gaussian_values_sorted, ranges):
    """FB pybind.cpp:179-208 (importance pass).  Returns (bucket_sum = 0, accum_weights_ptr (P,) f32,
    accum_weights_count (P,) i32, accum_max_count (P,) f32)."""
    dev = _device_of(splat_buffer)
    f = dict(device=dev)
    w = torch.empty(P, dtype=torch.float32, **f)
    cnt = torch.empty(P, dtype=torch.int32, **f)
    mx = torch.empty(P, dtype=torch.float32, **f)
    _lib.call("fgs_render_simp", int(P), int(num_rendered), int(width), int(height), _ptr(splat_buffer),
              _ptr(gaussian_keys_sorted), _ptr(gaussian_values_sorted), _ptr(ranges), _ptr(w), _ptr(cnt), _ptr(mx),
              _stream(dev))
    return 0, w, cnt, mx


def render_depth(P, num_rendered, width, height, splat_buffer, gaussian_keys_sorted, gaussian_values_sorted, ranges,
                 means3D, scales, rotations, proj_matrix, campos):
    """FB pybind.cpp:135-176 (depth pass).  Returns (out_pts (3,H,W), out_depth (1,H,W), accum_alpha (1,H,W),
    gidx (1,H,W) i32, discriminants (1,H,W))."""
    dev = _device_of(splat_buffer)
    H, W = int(height), int(width)
    f = dict(dtype=torch.float32, device=dev)
    out_pts = torch.empty((3, H, W), **f)
    out_depth = torch.empty((1, H, W), **f)
    accum_alpha = torch.empty((1, H, W), **f)
    gidx = torch.empty((1, H, W), dtype=torch.int32, device=dev)
    disc = torch.empty((1, H, W), **f)
    _lib.call("fgs_render_depth", int(P), int(num_rendered), W, H, _ptr(splat_buffer), _ptr(gaussian_keys_sorted),
              _ptr(gaussian_values_sorted), _ptr(ranges), _ptr(_f32("means3D", means3D, dev)),
              _ptr(_f32("scales", scales, dev)), _ptr(_f32("rotations", rotations, dev)),
              _ptr(_f32("proj_matrix", proj_matrix, dev)), _ptr(_f32("campos", campos, dev)), _ptr(out_pts),
              _ptr(out_depth), _ptr(accum_alpha), _ptr(gidx), _ptr(disc), _stream(dev))
    return out_pts, out_depth, accum_alpha, gidx, disc


def device_errors(dev: torch.device | None = None, clear: bool = True) -> int:
    """Reads (and clears) the library's device error word; synchronises the stream."""
    dev = dev or torch.device("cuda", torch.cuda.current_device())
    flags = C.c_int(0)
    _lib.call("fgs_device_errors", C.byref(flags), int(clear), _stream(dev))
    return int(flags.value)


ops = SimpleNamespace(preprocess=preprocess, sort_gaussian=sort_gaussian,
                      get_sort_buffer_size=get_sort_buffer_size, render_16x16=render_16x16, backward=backward,
                      adamUpdate=adamUpdate, render_simp=render_simp, render_depth=render_depth)


# ---------------------------------------------------------------------------------------------------------
# The vanilla 3DGS extension's entry points (gs_submodules/diff-gaussian-rasterization/ext.cpp:16-17,
# rasterize_points.h:18-59) over the same C ABI: vanilla tensor layouts (sh (P, 16, 3) with the DC term
# first, dL/dmeans2D (P, 3), dL/dsh (P, 16, 3)), FB's rasterization (bucket-granular stopping, ellipse tile
# test).  The three opaque buffers carry the forward state to the backward:
#   geomBuffer    float32 (P, 32): splat records;
#   binningBuffer int32 [sorted record ids (R) | tile ranges (2 T)];
#   imageBuffer   uint8 [image state | sample state | last contributor (H W) | final transmittance (H W)].
_ALIAS_CAP: dict = {}


def _align(v: int, a: int = 256) -> int:
    return (v + a - 1) // a * a


def _image_layout(R: int, W: int, H: int):
    mb, ib, sb = state_sizes(R, W, H, TILE, TILE, BUCKET)
    mb = max(mb, 1)
    sbytes = (mb + 1) * _SAMPLE_ROW
    off_smp = _align(ib)
    off_lc = _align(off_smp + sbytes)
    off_ts = _align(off_lc + 4 * W * H)
    return mb, ib, sbytes, off_smp, off_lc, off_ts, off_ts + 4 * W * H


def _split_sh(sh, dev):
    if sh is None or sh.numel() == 0:
        return torch.empty(0), torch.empty(0)
    sh = _f32("sh", sh, dev)
    return sh[:, :1].contiguous(), sh[:, 1:].contiguous()


def rasterize_gaussians(background, means3D, colors, opacity, scales, rotations, scale_modifier, cov3D_precomp,
                        viewmatrix, projmatrix, tan_fovx, tan_fovy, image_height, image_width, sh, degree, campos,
                        prefiltered, debug):
    """Vanilla RasterizeGaussiansCUDA (rasterize_points.h:18-37): returns
    (num_rendered, color (3, H, W), radii (P,), geomBuffer, binningBuffer, imageBuffer)."""
    if cov3D_precomp is not None and cov3D_precomp.numel():
        raise NotImplementedError("precomputed 3D covariances are not supported (FB needs scales and rotations)")
    dev = _device_of(means3D)
    P, W, H = int(means3D.size(0)), int(image_width), int(image_height)
    dc, rest = _split_sh(sh, dev)
    T = ((W + TILE - 1) // TILE) * ((H + TILE - 1) // TILE)
    geom = torch.empty((max(P, 1), 32), dtype=torch.float32, device=dev)
    curr = torch.zeros(1, dtype=torch.int32, device=dev)
    key = (dev.type, dev.index)
    cap = _ALIAS_CAP.get(key, 1 << 22)
    while True:
        keys_u = torch.empty(cap, dtype=torch.int64, device=dev)
        vals_u = torch.empty(cap, dtype=torch.int32, device=dev)
        tasks = torch.empty(cap, dtype=torch.int32, device=dev)
        curr.zero_()
        radii = preprocess(int(degree), means3D, colors, dc, rest, opacity, scales, rotations, scale_modifier, W, H,
                           TILE, TILE, campos, viewmatrix, projmatrix, tan_fovx, tan_fovy, 100.0, 0.01, keys_u,
                           vals_u, tasks, curr, 1.0, geom, None)
        R = int(curr.item())
        errors = device_errors(dev)
        if R < cap and not errors:
            break
        cap = max(2 * cap, 2 * R)  # pairs or large-footprint sub-tasks did not fit: grow and redo
        _ALIAS_CAP[key] = cap
    binning = torch.empty(R + 2 * T, dtype=torch.int32, device=dev)
    keys_s = torch.empty(max(R, 1), dtype=torch.int64, device=dev)
    tmp = torch.empty(int(_lib.load().fgs_sort_temp_bytes(max(R, 1))), dtype=torch.uint8, device=dev)
    s = _stream(dev)
    if R:
        _lib.call("fgs_sort", R, W, H, TILE, TILE, _ptr(tmp), tmp.numel(), _ptr(keys_u), _ptr(vals_u), _ptr(keys_s),
                  _ptr(binning), s)
    mb, ib, sbytes, off_smp, off_lc, off_ts, total = _image_layout(R, W, H)
    image = torch.empty(total, dtype=torch.uint8, device=dev)
    bg = _f32("background", background, dev)
    color = torch.empty((3, H, W), dtype=torch.float32, device=dev)
    base = image.data_ptr()
    _lib.call("fgs_render_fwd", P, R, W, H, TILE, TILE, BUCKET, _ptr(geom), _ptr(keys_s), _ptr(binning),
              binning.data_ptr() + 4 * R, _ptr(bg), _ptr(color), base + off_lc, base + off_ts, base, ib,
              base + off_smp, sbytes, mb, None, s)
    return R, color, radii, geom, binning, image


def rasterize_gaussians_backward(background, means3D, radii, colors, scales, rotations, scale_modifier,
                                 cov3D_precomp, viewmatrix, projmatrix, tan_fovx, tan_fovy, dL_dout_color, sh, degree,
                                 campos, geomBuffer, R, binningBuffer, imageBuffer, debug):
    """Vanilla RasterizeGaussiansBackwardCUDA (rasterize_points.h:39-59): returns
    (dL_dmeans2D (P, 3), dL_dcolors, dL_dopacity, dL_dmeans3D, dL_dcov3D, dL_dsh (P, 16, 3), dL_dscales,
    dL_drotations)."""
    if cov3D_precomp is not None and cov3D_precomp.numel():
        raise NotImplementedError("precomputed 3D covariances are not supported (FB needs scales and rotations)")
    dev = _device_of(means3D)
    P, R = int(means3D.size(0)), int(R)
    dL = _f32("dL_dout_color", dL_dout_color, dev)
    H, W = int(dL.size(1)), int(dL.size(2))
    dc, rest = _split_sh(sh, dev)
    M = rest.size(1) if rest.numel() else 0
    f = dict(dtype=torch.float32, device=dev)
    out = dict(dmean2D=torch.empty((P, 4), **f), dconic=torch.empty((P, 4), **f), dopac=torch.empty((P, 1), **f),
               dcolor=torch.empty((P, 3), **f), dmean3D=torch.empty((P, 3), **f), dcov3D=torch.empty((P, 6), **f),
               ddc=torch.empty((P, 1, 3), **f), dsh=torch.empty((P, M, 3), **f), dscale=torch.empty((P, 3), **f),
               drot=torch.empty((P, 4), **f))
    if P:
        mb, ib, sbytes, off_smp, off_lc, off_ts, total = _image_layout(R, W, H)
        if imageBuffer.numel() < total or binningBuffer.numel() < R:
            raise ValueError("imageBuffer / binningBuffer do not match num_rendered and the image size")
        base = imageBuffer.data_ptr()
        bg = _f32("background", background, dev)
        grad = torch.empty((P, 12), **f)
        s = _stream(dev)
        _lib.call("fgs_render_bwd", P, W, H, TILE, TILE, BUCKET, _ptr(binningBuffer), binningBuffer.data_ptr() + 4 * R,
                  _ptr(bg), _ptr(geomBuffer), base + off_ts, base + off_lc, base, base + off_smp, mb, _ptr(dL),
                  _ptr(grad), 0, s)
        _lib.call("fgs_preprocess_bwd", P, int(degree), int(M), _ptr(_f32("means3D", means3D, dev)), _ptr(radii),
                  _ptr(dc), _ptr(rest), _ptr(geomBuffer), _ptr(_f32("scales", scales, dev)),
                  _ptr(_f32("rotations", rotations, dev)), float(scale_modifier),
                  _ptr(_f32("viewmatrix", viewmatrix, dev)), _ptr(_f32("projmatrix", projmatrix, dev)), W, H,
                  float(tan_fovx), float(tan_fovy), _ptr(_f32("campos", campos, dev)), _ptr(grad),
                  _ptr(out["dmean2D"]), _ptr(out["dconic"]), _ptr(out["dopac"]), _ptr(out["dcolor"]),
                  _ptr(out["dmean3D"]), _ptr(out["dcov3D"]), _ptr(out["ddc"]), _ptr(out["dsh"]),
                  _ptr(out["dscale"]), _ptr(out["drot"]), 0, 0, 0, 0, s)
    dmeans2D = torch.zeros((P, 3), **f)
    dmeans2D[:, :2] = out["dmean2D"][:, :2]
    has_sh = sh is not None and sh.numel() != 0
    dsh = torch.cat([out["ddc"], out["dsh"]], dim=1) if has_sh else torch.empty(0, **f)
    return (dmeans2D, out["dcolor"], out["dopac"], out["dmean3D"], out["dcov3D"], dsh, out["dscale"], out["drot"])
