"""CPU tests of the C ABI: libfgs.so loads without a GPU, exports every
function include/fgs.h declares, and its host-only entry points behave."""
import ctypes as C
import re
from pathlib import Path

import pytest

import __graft_entry__
from fastergs_gb300 import _C, _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "fgs.h"


@pytest.fixture(scope="module")
def lib():
    __graft_entry__.build()
    return _lib.load()


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(fgs_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_status_strings_and_version(lib):
    assert lib.fgs_version().decode().startswith("fgs")
    for st in range(6):
        assert lib.fgs_status_string(st)
    assert b"unknown" in lib.fgs_status_string(99)


def test_sizing_helpers(lib):
    assert lib.fgs_sort_temp_bytes(0) > 0
    assert lib.fgs_sort_temp_bytes(1 << 20) > 12 * (1 << 20)
    # counted in composited sub-buckets (64 Gaussians for FB's 128), one
    # partially filled one per tile at most
    assert lib.fgs_max_buckets(1000, 256, 256, 16, 16, 128) == 16 + 256
    assert lib.fgs_max_buckets(1000, 256, 256, 16, 16, 64) == 16 + 256
    assert lib.fgs_max_buckets(1000, 256, 256, 16, 16, 32) == 32 + 256
    # other sizes: the fewest equal sub-buckets of <= 64 Gaussians that tile the bucket
    assert lib.fgs_max_buckets(1000, 256, 256, 16, 16, 96) == 21 + 256    # 2 x 48
    assert lib.fgs_max_buckets(1000, 256, 256, 16, 16, 65) == 77 + 256    # 5 x 13
    assert lib.fgs_max_buckets(1000, 256, 256, 16, 16, 97) == 1000 + 256  # prime: 97 x 1
    assert lib.fgs_max_buckets(10, 256, 256, 16, 16, 128) == 1 + 10
    ib, sb = C.c_size_t(0), C.c_size_t(0)
    assert lib.fgs_state_bytes(256, 256, 16, 16, 100, C.byref(ib), C.byref(sb)) == 0
    assert ib.value >= 3 * 4 * 256 * 256 and sb.value >= 100 * 256 * 16
    assert sb.value <= (100 + 1) * _C._SAMPLE_ROW


def test_bad_arguments_are_rejected_without_touching_the_gpu(lib):
    assert lib.fgs_preprocess(-1, 0, 0, *([None] * 7), 1.0, 16, 16, 16, 16, None, None, None, 1.0, 1.0, 100.0,
                              0.01, 1.0, None, None, 0, None, None, 0, None, 0, None, None, None, None) == 1
    assert lib.fgs_sort(-5, 256, 256, 16, 16, None, 0, None, None, None, None, None) == 1
    assert lib.fgs_sort(0, 256, 256, 16, 16, None, 0, None, None, None, None, None) == 0
    assert lib.fgs_render_fwd(1, 10, 256, 256, 16, 8, 128, *([None] * 9), 0, None, 0, 10, None, None) == 1
    assert lib.fgs_render_bwd(1, 256, 256, 16, 16, 0, *([None] * 8), 0, None, None, 0, None) == 1
    assert lib.fgs_adam_update(None, None, None, None, None, 0.1, 0.9, 0.999, 1e-8, 10, 0, None) == 1


def _cams(sizes):
    from fastergs_gb300 import _lib
    arr = (_lib.Camera * len(sizes))()
    for c, (w, h) in zip(arr, sizes):
        # device pointers are never dereferenced by the sizing call; any non-null value will do
        c.viewmatrix = c.projmatrix = c.campos = c.bg = 256
        c.width, c.height = w, h
        c.tan_fovx = c.tan_fovy = 0.5
        c.scale_modifier = c.mult = 1.0
    return arr


def _ws(P, sizes, cfg, pairs):
    import ctypes as C
    from fastergs_gb300 import _lib
    out = C.c_size_t(0)
    st = _lib.load().fgs_batch_workspace_bytes(P, len(sizes), _cams(sizes), C.byref(cfg), pairs, C.byref(out))
    return st, int(out.value)


def test_batch_workspace_sizing_and_validation():
    from fastergs_gb300 import _lib
    sizes = [(1297, 840), (640, 360), (1920, 1080)]
    fb = _lib.TuneConfig(128, 16, 16, 4, 0)
    st, small = _ws(100_000, sizes, fb, 1 << 20)
    assert st == 0 and small > 0
    st, big = _ws(100_000, sizes, fb, 1 << 22)
    assert st == 0 and big > small
    st, rec = _ws(100_000, sizes, _lib.TuneConfig(128, 16, 16, 4, 1), 1 << 22)
    assert st == 0 and rec < big  # one prefix per tile instead of per bucket
    st, b16 = _ws(100_000, sizes, _lib.TuneConfig(16, 8, 32, 2, 0), 1 << 22)
    assert st == 0 and b16 > big  # eight times the buckets
    for cfg in (_lib.TuneConfig(0, 16, 16, 4, 0), _lib.TuneConfig(129, 16, 16, 4, 0),
                _lib.TuneConfig(64, 8, 16, 4, 0), _lib.TuneConfig(64, 16, 16, 3, 0), _lib.TuneConfig(64, 16, 16, 4, 2),
                _lib.TuneConfig(64, 16, 16, 4, 0, -1)):
        assert _ws(1000, sizes, cfg, 1 << 20)[0] == 1  # FGS_ERR_BAD_ARG
    assert _ws(1000, [], fb, 1 << 20)[0] == 1
    assert _ws(1000, [(64, 64)] * 33, fb, 1 << 20)[0] == 1
    assert _ws(1000, sizes, fb, 1 << 30)[0] == 2  # FGS_ERR_CAPACITY: beyond the sort's 30-bit counts


def test_tuner_search_space_and_cache_key():
    from fastergs_gb300 import tune
    from fastergs_gb300.batched import TuneConfig
    space = tune.search_space(include_default=False)
    assert len(space) == 24 and len(set(space)) == 24
    assert TuneConfig() in tune.search_space() and len(tune.search_space()) == 25
    assert {c.bucket_size for c in space} == {16, 32, 64}
    assert {(c.block_x, c.block_y) for c in space} == {(16, 16), (8, 32)}
    assert {c.packet for c in space} == {1, 2, 4, 8}
    assert TuneConfig() == TuneConfig(128, 16, 16, 1, False)  # FB's fixed choice
    k1 = tune.cache_key(1_000_000, [(840, 1297), (360, 640)], 3, True)
    assert k1 == tune.cache_key(600_000, [(840, 1297), (360, 640)], 3, True)  # same power-of-two range
    assert k1 != tune.cache_key(1_000_000, [(840, 1297), (360, 640)], 3, False)
    assert k1 != tune.cache_key(3_000_000, [(840, 1297), (360, 640)], 3, True)


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors of fgs_camera, fgs_tune_config and fgs_adam_fused have the C layout."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    probe = tmp_path / "layout.c"
    fields = {"fgs_camera": (_lib.Camera, ["viewmatrix", "bg", "width", "mult"]),
              "fgs_tune_config": (_lib.TuneConfig, ["bucket_size", "recompute"]),
              "fgs_adam_fused": (_lib.AdamFused, ["param", "exp_avg", "exp_avg_sq", "lr", "lr_value", "eps", "b1",
                                                  "b2", "opacity_act", "scaling_act", "rotation_act"])}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "fgs.h"', "int main(void) {"]
    for name, (_, fs) in fields.items():
        lines.append(f'  printf("%zu\\n", sizeof({name}));')
        lines += [f'  printf("%zu\\n", offsetof({name}, {f}));' for f in fs]
    lines += ["  return 0;", "}"]
    probe.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(HEADER.parent), str(probe), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    want = []
    for name, (cls, fs) in fields.items():
        want.append(C.sizeof(cls))
        want += [getattr(cls, f).offset for f in fs]
    assert got == want


def test_fused_adam_entries_reject_bad_arguments(lib):
    a = _lib.AdamFused()
    s = None
    # P == 0 is a no-op; a missing description, moments or an unknown activation is BAD_ARG
    assert lib.fgs_preprocess_bwd_adam(0, 0, 0, None, None, None, None, None, None, None, 1.0, None, None, 8, 8, 0.5,
                                       0.5, None, None, C.byref(a), None, None, None, None, s) == 0
    dummy = C.c_void_p(256)
    args = [8, 0, 0, dummy, dummy, None, dummy, dummy, dummy, dummy, 1.0, dummy, dummy, 8, 8, 0.5, 0.5, dummy, dummy]
    assert lib.fgs_preprocess_bwd_adam(*args, None, None, None, None, None, s) == 1
    a.param[0] = 256  # xyz without moments
    assert lib.fgs_preprocess_bwd_adam(*args, C.byref(a), None, None, None, None, s) == 1
    a.exp_avg[0] = a.exp_avg_sq[0] = 512
    a.opacity_act = 7
    assert lib.fgs_preprocess_bwd_adam(*args, C.byref(a), None, None, None, None, s) == 1
    a.opacity_act = _lib.ACT["sigmoid"]
    a.param[3], a.exp_avg[3], a.exp_avg_sq[3] = 256, 512, 768  # sigmoid opacity without the activated opacities
    assert lib.fgs_preprocess_bwd_adam(*args[:7], None, *args[8:], C.byref(a), None, None, None, None, s) == 1
    a.param[5], a.exp_avg[5], a.exp_avg_sq[5] = 260, 512, 768  # misaligned rotation rows
    assert lib.fgs_preprocess_bwd_adam(*args, C.byref(a), None, None, None, None, s) == 1


def test_fused_adam_row_index_in_fp32_is_exact():
    """The fused step finds the Gaussian of f_rest element j of a 256-Gaussian block as
    floor((j + 1/2) / row) and floor((j + 7/2) / row) in FP32 (row = 3 M, M <= 16): equal to
    integer division for every row and element."""
    import numpy as np
    for row in range(3, 49):
        inv = np.float32(1) / np.float32(row)
        j = np.arange(256 * row, dtype=np.int64)
        for off in (0, 3):
            got = ((j.astype(np.float32) + np.float32(off + 0.5)) * inv).astype(np.int64)
            assert np.array_equal(got, (j + off) // row), row


def test_rect_row_index_in_fp32_is_exact():
    """The preprocess finds the tile row of candidate `local` of a small Gaussian's rectangle
    (area < 128 tiles, width w) as floor((local + 1/2) * fl(1 / w)) in FP32: equal to integer
    division for every width up to 255 and every local < 256."""
    import numpy as np
    j = np.arange(256, dtype=np.int64)
    for w in range(1, 256):
        inv = np.float32(1) / np.float32(w)
        got = ((j.astype(np.float32) + np.float32(0.5)) * inv).astype(np.int64)
        assert np.array_equal(got, j // w), w


def _declarations():
    """{name: (return type, [parameter declarations])} of every function include/fgs.h declares."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    text = re.sub(r"#[^\n]*", "", text)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(fgs_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text):
        params = [p.strip() for p in m.group(3).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(2)] = (" ".join(m.group(1).split()), params)
    return out


def test_ctypes_signatures_match_the_header_arity():
    decls = _declarations()
    assert set(decls) == set(_lib.SIGNATURES), set(decls) ^ set(_lib.SIGNATURES)
    for name, (ret, params) in decls.items():
        restype, argtypes = _lib.SIGNATURES[name]
        assert len(argtypes) == len(params), (name, len(argtypes), len(params))
        for p, a in zip(params, argtypes):
            ptr = "*" in p
            if ptr:
                assert a in (C.c_void_p, C.c_char_p) or hasattr(a, "_type_") and not isinstance(a._type_, str), \
                    (name, p, a)
            else:
                assert a not in (C.c_void_p,) or "void*" in p.replace(" ", ""), (name, p, a)
        if ret.endswith("*"):
            assert restype in (C.c_char_p, C.c_void_p), (name, ret)
        elif "size_t" in ret:
            assert restype == C.c_size_t, (name, ret)
        elif "int64_t" in ret:
            assert restype == C.c_int64, (name, ret)
        else:
            assert restype == C.c_int, (name, ret)
