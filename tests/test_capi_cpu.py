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
    # one partially filled bucket per tile at most
    assert lib.fgs_max_buckets(1000, 256, 256, 16, 16, 128) == 8 + 256
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
    assert lib.fgs_render_bwd(1, 256, 256, 16, 16, 0, *([None] * 8), 0, None, None, None) == 1
    assert lib.fgs_adam_update(None, None, None, None, None, 0.1, 0.9, 0.999, 1e-8, 10, 0, None) == 1
