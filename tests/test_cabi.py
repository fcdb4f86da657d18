"""The C-ABI library: loads without a GPU, exports every declared entry point,
and reports errors (not faults) when no device is present."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xgb.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:xgb_status|void|const char\*)\s+(xgb_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from xitils_gb300 import build
    path = build.build()
    return C.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert len(syms) >= 30
    assert "xgb_render" in syms and "xgb_scene_build" in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_defaults(lib):
    from xitils_gb300.api import IntegratorParamsC
    lib.xgb_version.restype = C.c_char_p
    assert b"sm_103a" in lib.xgb_version()
    p = IntegratorParamsC()
    lib.xgb_integrator_params_default(C.byref(p))
    assert (p.integrator, p.max_depth, p.rr_start) == (0, 0, 5)
    assert abs(p.rr_prob - 0.9) < 1e-7


def test_null_arguments_are_rejected(lib):
    lib.xgb_ctx_create.argtypes = [C.c_int, C.c_void_p]
    assert lib.xgb_ctx_create(0, None) == 1  # XGB_INVALID_ARG
    lib.xgb_render.argtypes = [C.c_void_p] * 3 + [C.c_uint32, C.c_uint32, C.c_void_p]
    assert lib.xgb_render(None, None, None, 0, 1, None) == 1
    lib.xgb_get_last_error.restype = C.c_char_p
    lib.xgb_get_last_error.argtypes = [C.c_void_p]
    assert lib.xgb_get_last_error(None) == b"null context"


def test_no_device_is_an_error_not_a_fault(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    lib.xgb_ctx_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    assert lib.xgb_ctx_create(0, C.byref(h)) == 3  # XGB_CUDA_ERROR
    from xitils_gb300 import api
    with pytest.raises(api.XgbError):
        api.Context(0)
