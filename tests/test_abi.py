"""CPU checks of the C ABI: the library exists (built here by build()),
exports every function include/ntgb300.h declares, and rejects bad
arguments before touching the GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ntgb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b((?:ntg|cuda)_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def native(pkg):
    from neko_top_gb300 import _native
    if not os.path.exists(_native.library_path()):
        import __graft_entry__ as ge
        ge._load_build_module().build()
    return _native


def test_header_declares_the_path():
    names = declared_functions()
    for must in ("ntg_plan_create", "ntg_ax_helm", "ntg_gs_op", "ntg_ksp_solve", "ntg_pc_jacobi_update",
                 "ntg_proj_pre_solving", "ntg_ramp_forward", "ntg_brinkman_compute", "cuda_col3_mask",
                 "cuda_cadd_mask", "cuda_sub3_mask", "cuda_invcol1_mask", "cuda_col2_mask"):
        assert must in names


def test_library_exports_every_declared_symbol(native):
    L = C.CDLL(native.library_path())
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding describes every one of them
    assert set(declared_functions()) <= set(native.SIGNATURES), set(declared_functions()) - set(native.SIGNATURES)


def test_argument_errors_are_reported_without_a_gpu(native):
    L = native.lib()
    h = C.c_void_p()
    st = L.ntg_plan_create(C.byref(h), 8, 1, None, None, None, None)
    assert st == native.NTG_ERR_INVALID
    assert b"lx" in L.ntg_last_error()
    st = L.ntg_plan_create(C.byref(h), 0, 8, None, None, None, None)
    assert st == native.NTG_ERR_INVALID
    assert L.ntg_ksp_create(None, 0, 10, 1e-10, 0.0, C.byref(h)) == native.NTG_ERR_INVALID
    assert L.ntg_proj_create(None, 4, C.byref(h)) == native.NTG_ERR_INVALID
    n = C.c_int64()
    assert L.ntg_mask_face_xmax(4, 3, 2, 8, None, C.byref(n), None) == 0 and n.value == 3 * 2 * 64
    assert L.ntg_version().startswith(b"ntgb300")
    lxs = (C.c_int * 16)()
    assert L.ntg_supported_lx(lxs, 16) >= 1 and 8 in list(lxs)
