"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares; host-side argument checks run without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest
from conftest import ROOT


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(modal_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def built_lib():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "modal-cmb_gb300"))
    import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "modal_gamma" in names and "modal_project" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_symbols() if not hasattr(built_lib, n)]
    assert missing == []


def test_python_binding_lists_every_symbol(mg):
    assert sorted(mg.EXPORTS) == sorted(n for n in declared_symbols() if n in mg.EXPORTS)
    assert set(declared_symbols()) <= set(mg.EXPORTS)


def test_argument_errors_without_gpu(built_lib, mg):
    L = mg.lib()
    x = np.zeros(4)
    assert L.modal_gl_nodes(0, x.ctypes.data_as(ctypes.c_void_p), x.ctypes.data_as(ctypes.c_void_p)) == 1
    assert b"n=0" in L.modal_last_error()
    assert L.modal_ctx_create(0, None) == 1
    assert L.modal_set_basis(None, 2, 10, 3, None) == 1
    n = ctypes.c_long()
    assert L.modal_tetrapyd_count(5, 2, ctypes.byref(n)) == 1
    assert L.modal_basis_prune(None, 4, None, 0, None, None, None) == 1
    assert L.modal_gamma_vjp(None, None, None) == 1
    assert L.modal_adjoint_residual(None, 1, None, None, None) == 1
    assert L.modal_lambda_min(None, None, None, None) == 1
    assert L.modal_project_batch(None, 1, None, 0, None) == 1
    assert L.modal_set_ortho(None, None, None) == 1
    assert L.modal_autotune(None, None) == 1
    assert L.modal_ctx_captures(None) == 0
    assert L.modal_set_basis_e(None, 2, 10, 3, None) == 1
    assert L.modal_gamma_pol(None, None, None, None) == 1
    assert L.modal_prim_points(5, 2, None, None) == 1
    assert L.modal_prim_ortho(None, 1, 10, 1.0, 3, None, 1, None, None) == 1
    assert L.modal_gamma_partial(None, 0, 0, 1, None) == 1
    assert L.modal_gamma_transfer_3d(None, 1.0, None) == 1


def test_tetrapyd_count_host_logic(built_lib, mg, orc):
    for lmin, lmax in [(2, 3), (2, 60), (3, 31), (2, 500)]:
        assert mg.tetrapyd_count(lmin, lmax) == orc.tetrapyd_count(lmin, lmax)
