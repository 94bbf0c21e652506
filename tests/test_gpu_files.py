"""The INI-driven GPU driver (modal_files.ortho_late): Gamma and the
orthogonalisation of the modes an INI file describes, written as raw FP64
files under the reference's names."""
import os

import numpy as np
import pytest

import modal_files as mf

pytestmark = pytest.mark.gpu


def test_ortho_late_driver_writes_reference_files(mg, tmp_path):
    lmax, N = 150, 35
    tri = mf._order_case2(N)  # set_terms_late case 2; the basis must cover its largest index
    P = int(tri.max()) + 1
    q, _, cl = mg.workload(lmax, P)
    ini = tmp_path / "run.ini"
    ini.write_text(f"[model]\ndirectory = {tmp_path}/\nT_lmin = 2\nT_lmax = {lmax}\n"
                   f"[basis]\nterms = {N}\norder_late = 2\n[old]\ngflag_pca = 1\n")
    bt = tmp_path / "basis_T.unf"
    mf.array_write(os.fspath(bt), q)
    mf.main(["ortho_late", os.fspath(ini), os.fspath(bt), "--pt", str(P)])
    names = mf.output_names(mf.read_ini(os.fspath(ini)))
    o = mf.array_read(names["orthol_TTT"], N * N).reshape(N, N)
    lam = mf.array_read(names["lambdal_TTT"], N * N).reshape(N, N)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tri)
        c.init_glint()
        g = c.gamma()
        o2, lam2, _, _ = c.orthogonalise(g)
    assert np.array_equal(o, o2) and np.array_equal(lam, lam2)
    assert os.path.basename(names["orthol_TTT"]) == f"orthol_TTT_2-{lmax}_2_{N}"
