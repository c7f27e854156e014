"""The C-ABI library loads without a GPU and exports every symbol include/gbint.h declares."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "gbint.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(gb_[a-z_]+)\(", text, re.M)))


def test_header_and_binding_agree():
    from diffrg_gb300 import capi

    assert declared_symbols() == sorted(capi.EXPORTS)


def test_library_exports_all_symbols(gblib):
    for name in declared_symbols():
        assert hasattr(gblib, name), name
    assert gblib.gb_version() == 1
    gblib.gb_status_string.restype = ctypes.c_char_p
    assert gblib.gb_status_string(0) == b"ok"
    assert gblib.gb_status_string(3) == b"HBM budget exceeded"


def test_no_device_is_reported_not_crashed(gblib):
    """Without a visible GPU the context constructor returns GB_ENODEV (the reference throws
    "No CUDA devices found!", integrator_4D_gpu.hh:81)."""
    import torch

    if torch.cuda.is_available():
        import pytest

        pytest.skip("a GPU is visible")
    h = ctypes.c_void_p()
    gblib.gb_ctx_create.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
    assert gblib.gb_ctx_create(0, 0, ctypes.byref(h)) == 6
