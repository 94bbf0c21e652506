"""Pins the torch float64 reference used by the adjoint tests (tests/adjoint_torch.py)
on the CPU: its Gamma against the oracle (itself pinned to the reference's
orthogonalisation_late.c), its projection against known answers, and its
autograd gradient against central finite differences."""
import numpy as np
import pytest
import torch
from conftest import rel_fro

import adjoint_torch as at

LMIN, LMAX, P, NMU = 2, 80, 4, 121


def _small(mg, orc):
    cl = mg.synthetic_cl(LMAX)
    qraw = mg.legendre_q(LMIN, LMAX, P)
    q = mg.weighted_q(qraw, cl, LMIN)
    tri = mg.mode_triples(P)
    mu, w = orc.gl_nodes(NMU)
    return cl, qraw, q, tri, mu, w


def _mode_shapes(qraw, tri, idx):
    """Separable single-term shapes equal to the (unweighted) modes tri[idx]."""
    out = []
    for m in idx:
        tab = np.zeros((1, 3, LMAX + 1))
        for a in range(3):
            tab[0, a, LMIN:] = qraw[:, tri[m][a]]
        out.append({"kind": 0, "tab": tab})
    return out


def test_torch_gamma_matches_oracle(mg, orc):
    cl, qraw, q, tri, mu, w = _small(mg, orc)
    pl = orc.legendre_table(mu, LMAX)
    M = orc.mij(pl, LMIN, LMAX, q)
    g_orc = orc.gamma(M, w, tri)
    pr = at.Problem(mu, w, LMIN, LMAX, tri, cl, None)
    g = pr.gamma(torch.tensor(q)).numpy()
    assert rel_fro(g, g_orc) <= 1e-13


def test_modes_as_shapes_project_exactly(mg, orc):
    # A shape equal to mode m has beta = Gamma[m], <S,S> = Gamma_mm and zero residual.
    cl, qraw, q, tri, mu, w = _small(mg, orc)
    idx = [0, 3, 7, len(tri) - 1]
    pr = at.Problem(mu, w, LMIN, LMAX, tri, cl, _mode_shapes(qraw, tri, idx))
    qt = torch.tensor(q)
    G = pr.gamma(qt).numpy()
    beta, n2 = pr.beta_norm2(qt)
    assert rel_fro(beta.numpy(), G[idx]) <= 1e-13
    assert np.max(np.abs(n2.numpy() - G[idx, idx]) / G[idx, idx]) <= 1e-13
    assert abs(pr.objective(qt).item()) <= 1e-12


def test_torch_gradient_matches_finite_differences(mg, orc):
    cl, qraw, q, tri, mu, w = _small(mg, orc)
    shapes = mg.separable_shapes(LMAX, 3, 7, 1, 2)
    pr = at.Problem(mu, w, LMIN, LMAX, tri, cl, shapes)
    qt = torch.tensor(q, requires_grad=True)
    pr.objective(qt).backward()
    g = qt.grad.numpy()
    rng = np.random.default_rng(1)
    for _ in range(3):
        d = rng.standard_normal(q.shape) * np.abs(q).max()
        h = 1e-6
        jp = pr.objective(torch.tensor(q + h * d)).item()
        jm = pr.objective(torch.tensor(q - h * d)).item()
        fd = (jp - jm) / (2 * h)
        an = float(np.sum(g * d))
        assert abs(fd - an) <= 1e-6 * abs(an) + 1e-12


def test_bspline_basis(mg):
    B = mg.bspline_matrix(2, 1000, 64)
    assert B.shape == (999, 64)
    assert np.all(B >= -1e-15)
    assert np.max(np.abs(B.sum(1) - 1.0)) <= 1e-14
    # each cubic B-spline spans at most 4 knot intervals
    support = (B > 0).sum(0)
    assert support.max() <= 4 * (998 // 61 + 2)
    C, Bw, tri, cl = mg.bspline_workload(1000, 12, 64, seed=4)
    assert C.shape == (12, 64) and Bw.shape == (999, 64) and tri.shape == (364, 3)
