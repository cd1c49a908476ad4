"""CPU tests of the C ABI: the library builds, loads, exports every entry point
declared in include/pointrix_gb300.h with ctypes argument and return types
that match the prototypes, and rejects bad arguments before any
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


def _prototypes():
    """{name: (return type, [parameter types])} of every prototype in the header."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for ret, name, args in re.findall(
            r"([A-Za-z_][A-Za-z0-9_ *]*?)\b(pgb_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        params = []
        for a in args.split(","):
            a = " ".join(a.split())
            if a and a != "void":
                params.append(re.sub(r"\s*\b[A-Za-z_][A-Za-z0-9_]*$", "", a).replace(" *", "*"))
        out[name] = (" ".join(ret.split()), params)
    return out


_SCALARS = {"int": C.c_int, "int64_t": C.c_int64, "float": C.c_float, "double": C.c_double,
            "size_t": C.c_size_t}
_POINTEES = {"size_t*": C.c_size_t, "int64_t*": C.c_int64,
             "const pgb_adam_segment*": _lib.AdamSegment}
_RETURNS = {"int": C.c_int, "int64_t": C.c_int64, "size_t": C.c_size_t, "const char*": C.c_char_p}


def test_ctypes_signatures_match_the_header_prototypes():
    """Each bound argument has the C type of its parameter (a wrong width
    would pass a corrupted value to the library), and each return type is
    read at its declared width."""
    protos = _prototypes()
    assert set(protos) == set(declared_functions())
    for name, (ret, params) in protos.items():
        bound = _lib.SIGNATURES[name]
        assert len(bound) == len(params), (name, len(bound), len(params))
        for i, (p, b) in enumerate(zip(params, bound)):
            if p.endswith("*"):
                want = _POINTEES.get(p)
                ok = b is C.c_void_p or (want is not None and b is C.POINTER(want))
            else:
                ok = b is _SCALARS[p]
            assert ok, f"{name} parameter {i}: header {p!r}, bound {b}"
        assert _lib._RESTYPES.get(name, C.c_int) is _RETURNS[ret], (name, ret)


_SIZE_QUERIES = {"pgb_status_string", "pgb_abi_version", "pgb_camera_grad_scratch_bytes",
                 "pgb_blend_record_floats", "pgb_blend_grad_record_floats",
                 "pgb_sh_rgb_scratch_floats", "pgb_sh_rgb_views_scratch_floats",
                 "pgb_l1_l2_loss_scratch_doubles", "pgb_ssim_scratch_doubles",
                 "pgb_sort_scratch_bytes", "pgb_blend_batches",
                 "pgb_camera_grad_views_scratch_bytes", "pgb_blend_batches_h",
                 "pgb_band_lists_scratch_bytes"}


def test_every_compute_entry_rejects_null_buffers():
    """Null buffers with a non-empty problem (16 of everything, 0.5 for
    every float) are refused with PGB_ERR_INVALID before any CUDA call, by
    every entry point that launches work."""
    import torch

    if torch.cuda.is_available():
        import pytest
        pytest.skip("argument checks are exercised where no device can be reached")
    lib = _lib.lib()
    launching = sorted(set(_lib.SIGNATURES) - _SIZE_QUERIES)
    assert len(launching) >= 40
    for name in launching:
        args = [None if (t is C.c_void_p or issubclass(t, C._Pointer)) else
                (0.5 if t in (C.c_float, C.c_double) else 16) for t in _lib.SIGNATURES[name]]
        assert getattr(lib, name)(*args) == 1, name


def test_blend_variant_list_is_sized_by_its_own_count():
    """pgb_blend_batches(backward, NULL) returns the count; the list then
    fits a buffer of exactly that size (the Python layer sizes it so)."""
    lib = _lib.lib()
    for backward in (0, 1):
        cnt = lib.pgb_blend_batches(backward, None)
        assert cnt >= 2
        buf = (C.c_int32 * cnt)()
        assert lib.pgb_blend_batches(backward, buf) == cnt
        assert len(set(buf)) == cnt
    from pointrix_gb300 import ops
    assert len(ops._blend_batches(1)) == lib.pgb_blend_batches(1, None)
