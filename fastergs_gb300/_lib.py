"""ctypes binding of libfgs.so (the C ABI declared in include/fgs.h).

The library is the product: there is no CPU or PyTorch fallback.  Loading
fails loudly when libfgs.so is missing; ``fastergs_gb300.build.build()``
compiles it for sm_103a.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

_LIB = None
_LOCK = threading.Lock()

vp, i32, i64, f32, sz = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_size_t
u32p = C.POINTER(C.c_uint32)


class Camera(C.Structure):
    """fgs_camera: one view of a batched frame (device pointers, host struct)."""
    _fields_ = [("viewmatrix", vp), ("projmatrix", vp), ("campos", vp), ("bg", vp), ("width", i32),
                ("height", i32), ("tan_fovx", f32), ("tan_fovy", f32), ("scale_modifier", f32), ("mult", f32)]


class TuneConfig(C.Structure):
    """fgs_tune_config: bucket size, tile shape and packet width of a launch."""
    _fields_ = [("bucket_size", i32), ("block_x", i32), ("block_y", i32), ("packet", i32), ("recompute", i32),
                ("chain", i32)]


ADAM_GROUPS = ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation")  # FGS_ADAM_* order
ACT = {"identity": 0, "sigmoid": 1, "exp": 2, "normalize": 3}  # FGS_ACT_*


class AdamFused(C.Structure):
    """fgs_adam_fused: raw parameters, moments and step sizes of the fused sparse Adam."""
    _fields_ = [("param", vp * 6), ("exp_avg", vp * 6), ("exp_avg_sq", vp * 6), ("lr", vp), ("lr_value", f32 * 6), ("eps", f32 * 6),
                ("b1", f32), ("b2", f32), ("opacity_act", i32), ("scaling_act", i32), ("rotation_act", i32)]


camp, tunep, adamp = C.POINTER(Camera), C.POINTER(TuneConfig), C.POINTER(AdamFused)

# name: (restype, argtypes) -- mirrors include/fgs.h
SIGNATURES = {
    "fgs_status_string": (C.c_char_p, [i32]),
    "fgs_version": (C.c_char_p, []),
    "fgs_device_errors": (i32, [C.POINTER(C.c_int), i32, vp]),
    "fgs_selftest_wait": (i32, [vp, vp]),
    "fgs_read_counts": (i32, [vp, vp, vp, vp]),
    "fgs_preprocess": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, f32, i32, i32, i32, i32, vp, vp, vp,
                             f32, f32, f32, f32, f32, vp, vp, i64, vp, vp, i64, vp, i64, vp, vp, vp, vp]),
    "fgs_sort_temp_bytes": (sz, [i64]),
    "fgs_sort": (i32, [i64, i32, i32, i32, i32, vp, sz, vp, vp, vp, vp, vp]),
    "fgs_sort_noalloc": (i32, [i64, i32, i32, i32, i32, vp, vp, vp, vp, vp]),
    "fgs_tile_ranges": (i32, [i64, i32, vp, vp, vp]),
    "fgs_max_buckets": (i64, [i64, i32, i32, i32, i32, i32]),
    "fgs_state_bytes": (i32, [i32, i32, i32, i32, i64, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "fgs_render_fwd": (i32, [i32, i64, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, sz, vp, sz,
                             i64, u32p, vp]),
    "fgs_render_bwd": (i32, [i32, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, i64, vp, vp, i32, vp]),
    "fgs_preprocess_bwd": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, f32, vp, vp, i32, i32, f32, f32, vp,
                                 vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "fgs_preprocess_bwd_adam": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, f32, vp, vp, i32, i32, f32, f32,
                                      vp, vp, adamp, vp, vp, vp, vp, vp]),
    "fgs_densify_stats": (i32, [i32, vp, vp, vp, vp, vp, vp, vp]),
    "fgs_ssim_fwd": (i32, [i32, i32, i32, f32, f32, vp, vp, vp, vp, vp, vp, vp]),
    "fgs_ssim_bwd": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
    "fgs_l1_dssim_scratch_bytes": (sz, [i32, i32, i32]),
    "fgs_l1_dssim": (i32, [i32, i32, i32, f32, vp, vp, vp, sz, vp, vp, vp, vp]),
    "fgs_render_simp": (i32, [i32, i64, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
    "fgs_render_depth": (i32, [i32, i64, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "fgs_adam_update": (i32, [vp, vp, vp, vp, vp, f32, f32, f32, f32, C.c_uint32, C.c_uint32, vp]),
    "fgs_batch_workspace_bytes": (i32, [i32, i32, camp, tunep, i64, C.POINTER(C.c_size_t)]),
    "fgs_render_batched_fwd": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, i32, camp, tunep, i64, vp, sz,
                                     vp, vp, vp]),
    "fgs_render_batched_bwd": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, i32, camp, tunep, i64, vp, sz, vp, vp,
                                     vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "fgs_render_batched_bwd_adam": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, i32, camp, tunep, i64, vp, sz, vp,
                                          vp, adamp, vp, vp, vp, vp, vp]),
    "fgs_tune_grad_bytes": (sz, [i32, i32]),
    "fgs_tune": (i32, [i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, i32, camp, tunep, i32, i64, vp, sz, vp, vp, vp,
                       vp, sz, i32, C.POINTER(C.c_int), C.POINTER(C.c_float), vp]),
    "fgs_batch_status": (i32, [i32, i32, camp, tunep, i64, vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), vp]),
    "fgs_batch_offsets": (i32, [i32, i32, camp, tunep, i64, C.POINTER(C.c_int64), i32]),
    "fgs_peak_fp32": (i32, [C.POINTER(C.c_double), vp]),
    "fgs_peak_fp32x2": (i32, [C.POINTER(C.c_double), vp]),
    "fgs_peak_ex2": (i32, [C.POINTER(C.c_double), vp]),
    "fgs_kernel_timer": (i32, [i32, i32]),
    "fgs_kernel_timer_read": (i32, [i32, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
}

# Kernel ids of fgs_kernel_timer (include/fgs.h).
KERNELS = {"preprocess": 0, "preprocess_large": 1, "sort_hist": 2, "sort_pass": 3, "tile_ranges": 4,
           "bucket_setup": 5, "render_fwd": 6, "empty_tiles": 7, "render_bwd": 8, "preprocess_bwd": 9,
           "loss": 10, "render_simp": 11, "render_depth": 12, "read_counts": 13,
           "bwd_list": 14, "deep_merge": 15, "zero": 16}


class FgsError(RuntimeError):
    """A C-ABI call returned a non-OK fgs_status."""

    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed: {msg} (status {status})")
        self.status = status


def lib_path() -> Path:
    return _build.LIB


def load() -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is None:
            p = lib_path()
            if not p.exists():
                raise ImportError(
                    f"{p} is missing: build the CUDA library first (python -m fastergs_gb300.build); "
                    "this package has no CPU fallback")
            lib = C.CDLL(str(p))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _LIB = lib
    return _LIB


def check(fn: str, status: int) -> None:
    if status != 0:
        msg = load().fgs_status_string(status).decode()
        raise FgsError(fn, status, msg)


def call(name: str, *args):
    st = getattr(load(), name)(*args)
    check(name, st)
    return st


def kernel_timers(enable: bool, names=None) -> None:
    """Turn per-kernel event timing on or off (all kernels by default)."""
    for n in names or KERNELS:
        call("fgs_kernel_timer", KERNELS[n], int(enable))


def read_kernel_timers(names=None) -> dict:
    """{name: (total_ms, launches)} since the previous read; synchronises."""
    out = {}
    for n in names or KERNELS:
        ms, cnt = C.c_double(0.0), C.c_int(0)
        call("fgs_kernel_timer_read", KERNELS[n], C.byref(ms), C.byref(cnt))
        out[n] = (float(ms.value), int(cnt.value))
    return out
