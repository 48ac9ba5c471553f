"""The C ABI library: it loads, exports every function include/rt_gb300.h declares, and
rejects bad input without touching a GPU."""
import ctypes as C
import os
import re

import pytest

import raytrace_gb300 as rt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "rt_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(rt_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_exports_every_declared_symbol():
    lib = C.CDLL(rt.LIB_PATH)
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(rt._SIGS)


def test_version():
    assert rt.lib.rt_version() == 1


def test_invalid_arguments_are_rejected():
    assert rt.lib.rt_ctx_create(0, None) == rt.RT_ERR_INVALID
    assert rt.lib.rt_render(None, 0, 0, None) == rt.RT_ERR_INVALID
    assert rt.lib.rt_scenegen(9, 0, C.byref(C.c_void_p())) == rt.RT_ERR_INVALID
    assert rt.lib.rt_scenegen_small(1, -1, 0, 8, 8, 0, C.byref(C.c_void_p())) == rt.RT_ERR_INVALID


def test_no_gpu_is_an_error_not_a_fallback():
    n = C.c_int()
    cudart = None
    try:
        # this container has no GPU: creating a context must fail with RT_ERR_CUDA
        h = C.c_void_p()
        rc = rt.lib.rt_ctx_create(0, C.byref(h))
        if rc == 0:
            rt.lib.rt_ctx_destroy(h)
            pytest.skip("a GPU is present")
        assert rc == rt.RT_ERR_CUDA
    finally:
        del n, cudart
