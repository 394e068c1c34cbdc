"""C ABI checks that need no GPU: the library builds, loads, and exports every
function include/sfwi_gb300.h declares; host-only entry points behave like the
reference; argument errors are reported, not crashed on."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from sfwi_gb300 import build, _lib
    build.build()
    return _lib.load()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "sfwi_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sfwi_\w+)\s*\(", src)))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for n in ("sfwi_create", "sfwi_gpu_buffer_vpvs", "sfwi_gpu_buffer_m", "sfwi_buffer_vpvs_htod",
              "sfwi_record_copy_to_gpu", "sfwi_image_singleshot", "sfwi_imagebuffer_resettozero", "sfwi_ot",
              "sfwi_ot_power", "sfwi_ot_alltrace", "sfwi_normalize"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from sfwi_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_normalize_matches_reference(lib):
    """normalize (sfwi-stage1/main.cpp:24-32): divide by max |x| of the gather."""
    rng = np.random.default_rng(0)
    a = rng.standard_normal((7, 33)).astype(np.float32)
    ref = a / np.max(np.abs(a))
    import sfwi_gb300 as sg
    out = sg.normalize(a.copy())
    assert np.array_equal(out, ref.astype(np.float32))


def test_create_reports_errors_without_crashing(lib):
    h = C.c_void_p()
    sou = np.zeros(10, np.float32)
    fp = sou.ctypes.data_as(C.POINTER(C.c_float))
    # nop != 4 is rejected before any device work
    rc = lib.sfwi_create(C.byref(h), 1, fp, 10.0, 10.0, 1e-3, 60, 60, 20, 20, 1, 20, 10, 2, 5)
    assert rc == -1 and b"nop" in lib.sfwi_last_error()
    rc = lib.sfwi_create(C.byref(h), 3, fp, 10.0, 10.0, 1e-3, 60, 60, 20, 20, 1, 20, 10, 4, 5)
    assert rc == -1
    rc = lib.sfwi_create(C.byref(h), 1, fp, 10.0, 10.0, 1e-3, 60, 61, 20, 20, 1, 20, 10, 4, 5)
    assert rc == -1 and b"nzpml" in lib.sfwi_last_error()
    # valid arguments: succeeds on a GPU host, reports "no CUDA device" elsewhere
    rc = lib.sfwi_create(C.byref(h), 1, fp, 10.0, 10.0, 1e-3, 60, 60, 20, 20, 1, 20, 10, 4, 5)
    if rc == 0:
        assert lib.sfwi_destroy(h) == 0
    else:
        assert rc == -5


def test_ot_rejects_bad_arguments(lib):
    m = C.c_double(0)
    assert lib.sfwi_ot(None, None, None, None, None, None, 10, 1, 1e-3, C.byref(m)) == -1


def test_null_handle_is_an_error(lib):
    assert lib.sfwi_image_singleshot(None, None) == -1
    assert lib.sfwi_destroy(None) == 0


def test_pinned_cache_limit_needs_no_device(lib):
    """sfwi_set_pinned_cache only sets a host-side limit (and frees cached
    blocks above it): callable without a GPU"""
    assert lib.sfwi_set_pinned_cache(1 << 30) == 0
    assert lib.sfwi_set_pinned_cache(0) == 0


def test_handle_calls_refuse_a_null_handle(lib):
    for rc in (lib.sfwi_set_cpu_mem(None, 1, 10), lib.sfwi_strip_bytes(None, None, None),
               lib.sfwi_hessian_vector(None, None, None, None, None)):
        assert rc != 0
