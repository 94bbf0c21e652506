"""Polarised Gamma (TTE, TEE, EEE) on the GPU against the reference's own
calculate_orthol with do_polarisation (golden) and the oracle."""
import os
import sys

import numpy as np
import pytest
from conftest import rel_fro, rel_max

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import pol_inputs  # noqa: E402

pytestmark = pytest.mark.gpu


def _ctx(mg, lmaxT, lmaxE, lminE):
    cl, qT, qE, ttt, tte, tee, eee = pol_inputs(lmaxT, lmaxE, lminE)
    c = mg.Context(0)
    c.set_basis(2, lmaxT, qT)
    c.set_modes(ttt)
    c.set_basis_e(lminE, lmaxE, qE)
    c.set_modes_pol(tte, tee, eee)
    return c, (cl, qT, qE, ttt, tte, tee, eee)


def test_pol_gamma_vs_reference(mg, golden):
    g = golden("gamma_pol")
    lmaxT, lmaxE, lminE = (int(v) for v in g["dims"])
    c, _ = _ctx(mg, lmaxT, lmaxE, lminE)
    with c:
        c.set_gl(g["nodes"], g["weights"])
        c.init_glint()
        gT = c.gamma()
        tte, tee, eee = c.gamma_pol()
        for got, want in zip((gT, tte, tee, eee), g["gamma"]):
            assert rel_fro(got, want) <= 1e-12 and rel_max(got, want) <= 1e-12
        r = c.orthol_pair(3, 11, all_four=True)
        assert np.allclose(r, g["gamma"][:, 3, 11], rtol=1e-12, atol=0)


def test_pol_gamma_own_nodes_vs_oracle(mg, orc):
    lmaxT, lmaxE, lminE = 70, 90, 2
    c, (cl, qT, qE, ttt, tte, tee, eee) = _ctx(mg, lmaxT, lmaxE, lminE)
    with c:
        c.init_glint()
        mu, w = c.get_gl()
        assert mu.size == 3 * lmaxE // 2 + 1  # the quadrature covers max(lmax_T, lmax_E)
        got = c.gamma_pol()
    pl = orc.legendre_table(mu, lmaxE)
    MT = orc.mij(np.ascontiguousarray(pl[:, :lmaxT + 1]), 2, lmaxT, qT)
    ME = orc.mij(pl, lminE, lmaxE, qE)
    want = orc.gamma_pol(MT, ME, w, tte, tee, eee)
    for a, b in zip(got, want):
        assert rel_max(a, b) <= 1e-12


def test_pol_argument_checks(mg):
    c, (cl, qT, qE, ttt, tte, tee, eee) = _ctx(mg, 50, 60, 3)
    with c:
        bad = tte.copy()
        bad[0, 2] = 4  # E index outside P_E
        with pytest.raises(mg.ModalError):
            c.set_modes_pol(bad, tee, eee)
        c.set_modes(ttt)  # a new TTT list drops the polarised one
        with pytest.raises(mg.ModalError):
            c.gamma_pol()


def test_pol_transfer_gamma_vs_reference(mg, golden):
    from make_golden import pol_transfer_inputs
    g = golden("gamma_transfer_pol")
    d = pol_transfer_inputs()
    with mg.Context(0) as c:
        c.set_basis(2, d["lmax"], d["qT"])
        c.set_modes(d["ttt"])
        c.set_spectrum(d["cl_total"])
        c.set_basis_e(d["lminE"], d["lmaxE"], d["qE"])
        c.set_modes_pol(d["tte"], d["tee"], d["eee"])
        c.set_gl(g["nodes"], g["weights"])
        c.set_transfer(d["xvec"], d["qtT"], d["prim"])
        c.set_transfer_pol(d["qtE"], d["spec9"], d["fsky_t"], d["fsky_e"])
        ttt = c.gamma_transfer(d["dphi"])
        got = c.gamma_transfer_pol(d["dphi"])
    assert rel_max(ttt, g["gamma"][0]) <= 1e-12
    for f in range(3):
        assert rel_fro(got[f], g["gamma"][f + 1]) <= 1e-12 and rel_max(got[f], g["gamma"][f + 1]) <= 1e-12
