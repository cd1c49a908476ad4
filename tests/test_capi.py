"""CPU tests of the C ABI: the library builds, loads, exports every entry point
declared in include/pointrix_gb300.h, and rejects bad arguments before any
CUDA call.  No kernel is launched."""
import ctypes as C
import re
from pathlib import Path

from pointrix_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "pointrix_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(pgb_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = _lib.lib()
    names = declared_functions()
    assert len(names) >= 17
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_status_strings_and_version():
    lib = _lib.lib()
    assert lib.pgb_abi_version() == 1
    assert lib.pgb_status_string(0) == b"ok"
    assert b"wait" in lib.pgb_status_string(4)


def test_invalid_arguments_rejected_without_launch():
    lib = _lib.lib()
    assert lib.pgb_compute_sh_forward(None, -1, 16, 48, 1, 3, None, None, None) == 1
    assert lib.pgb_compute_sh_forward(None, 10, 5, 15, 1, 3, None, None, None) == 1
    assert lib.pgb_project_point_forward(None, 10, None, None, 0, 10, 0.2, 1.3, None, None, None) == 1
    assert lib.pgb_blend_record_floats(7) == 16
    assert lib.pgb_blend_record_floats(3) == 12
    assert lib.pgb_blend_record_floats(26) == 36
    assert lib.pgb_blend_grad_record_floats(7) == 16
    assert lib.pgb_blend_grad_record_floats(26) == 32
    assert lib.pgb_blend_record_floats(27) == -1
    bn, bk = C.c_size_t(0), C.c_size_t(0)
    assert lib.pgb_sort_scratch_bytes(1000, 5000, 64, 64, C.byref(bn), C.byref(bk)) == 0
    assert bn.value >= 16 * 1000
    # K-sized pair buffers by tile passes: none for one pass (16 tiles), one
    # (key, value) pair buffer for two, two for three
    one = bk.value
    assert lib.pgb_sort_scratch_bytes(1000, 5000, 1600, 1060, C.byref(bn), C.byref(bk)) == 0
    two = bk.value
    assert lib.pgb_sort_scratch_bytes(1000, 5000, 16 * 300000, 16, C.byref(bn), C.byref(bk)) == 0
    three = bk.value
    assert two - one >= 8 * 5000 and three - two >= 8 * 5000
    assert lib.pgb_sort_scratch_bytes(-1, 0, 64, 64, C.byref(bn), C.byref(bk)) == 1
    # scratch too small is refused before any CUDA call
    assert lib.pgb_sort_gaussian_begin(None, None, None, 1000, 64, 64, None, 0, None, None) == 1
