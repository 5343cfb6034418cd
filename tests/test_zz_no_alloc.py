"""fgs_sort_noalloc: the sort entry point for callers that cannot allocate
device memory when they sort (code inside a memory pool or arena it does not
own, hosts that forbid allocation after start-up, real-time loops that must
not stall on cudaMalloc).  Its scratch is a static device array inside the
library, so it must give the same result as fgs_sort with caller scratch,
call after call.

Kept in a file that pytest collects last; it passes alone in a fresh process
and after the other tests.
"""
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest
import torch

from fastergs_gb300 import _C, _lib

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 20  # FGS_SORT_NOALLOC_MAX_PAIRS in include/fgs.h


def _keys(K, W, H, seed):
    T = ((W + 15) // 16) * ((H + 15) // 16)
    rng = np.random.default_rng(seed)
    tiles = rng.integers(0, T, K, dtype=np.uint64)
    depth = rng.choice(rng.uniform(0.2, 50.0, size=max(K // 8, 1)).astype(np.float32), size=K).view(np.uint32)
    return (tiles << np.uint64(32)) | depth.astype(np.uint64), rng.permutation(K).astype(np.uint32)


def _run(fn, K, W, H, keys, vals, dev):
    k_in = torch.tensor(keys.view(np.int64), device=dev)
    v_in = torch.tensor(vals.view(np.int32), device=dev)
    k_out = torch.full((K,), -1, dtype=torch.int64, device=dev)
    v_out = torch.full((K,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    if fn == "fgs_sort":
        tmp = torch.empty(int(_lib.load().fgs_sort_temp_bytes(K)), dtype=torch.uint8, device=dev)
        _lib.call("fgs_sort", K, W, H, 16, 16, tmp.data_ptr(), tmp.numel(), k_in.data_ptr(), v_in.data_ptr(),
                  k_out.data_ptr(), v_out.data_ptr(), stream)
    else:
        _lib.call("fgs_sort_noalloc", K, W, H, 16, 16, k_in.data_ptr(), v_in.data_ptr(), k_out.data_ptr(),
                  v_out.data_ptr(), stream)
    torch.cuda.synchronize()
    assert _C.device_errors(dev) == 0
    return k_out.cpu().numpy().view(np.uint64), v_out.cpu().numpy().view(np.uint32)


def test_sort_noalloc_matches_sort_on_consecutive_calls(cuda_device):
    # Two calls in a row share (and reuse) the library's scratch array; the
    # second has a different size, tile count and seed.
    for K, (W, H), seed in [(700_001, (1297, 840), 1), (MAX_PAIRS, (3840, 2160), 2)]:
        keys, vals = _keys(K, W, H, seed)
        ka, va = _run("fgs_sort", K, W, H, keys, vals, cuda_device)
        kb, vb = _run("fgs_sort_noalloc", K, W, H, keys, vals, cuda_device)
        np.testing.assert_array_equal(kb, ka)
        np.testing.assert_array_equal(vb, va)
        order = np.argsort(keys, kind="stable")
        np.testing.assert_array_equal(kb, keys[order])


def test_sort_noalloc_rejects_more_pairs_than_its_scratch_holds(cuda_device):
    with pytest.raises(_lib.FgsError, match="too small"):
        _lib.call("fgs_sort_noalloc", MAX_PAIRS + 1, 256, 256, 16, 16, 0, 0, 0, 0,
                  torch.cuda.current_stream().cuda_stream)


# A process of its own (no torch): sorts through fgs_sort_noalloc, resets the
# device (which destroys the context and the library's static array with it),
# and sorts again in the new context.  The second call must find the array's
# new address instead of reusing the first context's.
_RESET_CHILD = textwrap.dedent("""
    import ctypes as C, sys
    import numpy as np
    fgs = C.CDLL(sys.argv[1])
    rt = C.CDLL("libcudart.so.13")
    vp = C.c_void_p
    rt.cudaMalloc.argtypes = [C.POINTER(vp), C.c_size_t]
    rt.cudaMemcpy.argtypes = [vp, vp, C.c_size_t, C.c_int]
    fgs.fgs_sort_noalloc.argtypes = [C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp]
    def check(e, what):
        if e != 0:
            raise SystemExit(f"{what}: error {e}")
    def sort_once(seed):
        rng = np.random.default_rng(seed)
        K, W, H = 300_001, 1297, 840
        T = ((W + 15) // 16) * ((H + 15) // 16)
        keys = (rng.integers(0, T, K, dtype=np.uint64) << np.uint64(32)) | rng.integers(
            0x3e000000, 0x42000000, K, dtype=np.uint64)
        vals = rng.permutation(K).astype(np.uint32)
        bufs = []
        for n in (8 * K, 4 * K, 8 * K, 4 * K):
            p = vp()
            check(rt.cudaMalloc(C.byref(p), n), "cudaMalloc")
            bufs.append(p)
        check(rt.cudaMemcpy(bufs[0], keys.ctypes.data, 8 * K, 1), "upload keys")
        check(rt.cudaMemcpy(bufs[1], vals.ctypes.data, 4 * K, 1), "upload values")
        check(fgs.fgs_sort_noalloc(K, W, H, 16, 16, bufs[0], bufs[1], bufs[2], bufs[3], None), "fgs_sort_noalloc")
        check(rt.cudaDeviceSynchronize(), "synchronize")
        ko, vo = np.empty(K, np.uint64), np.empty(K, np.uint32)
        check(rt.cudaMemcpy(ko.ctypes.data, bufs[2], 8 * K, 2), "download keys")
        check(rt.cudaMemcpy(vo.ctypes.data, bufs[3], 4 * K, 2), "download values")
        order = np.argsort(keys, kind="stable")
        if not (np.array_equal(ko, keys[order]) and np.array_equal(vo, vals[order])):
            raise SystemExit(f"seed {seed}: sorted output differs from a stable sort")
    sort_once(1)
    check(rt.cudaDeviceReset(), "cudaDeviceReset")
    sort_once(2)
    print("ok")
""")


def test_sort_noalloc_after_device_reset(cuda_device):
    lib = Path(_lib.load()._name)
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, str(lib)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
