"""GPU greedy basis pruning (basis_optimisation_mpi.c:184-337) against the
reference's own driver (golden orders) and the numpy restatement, and the
smallest-eigenvalue objective's gradient against torch float64 autograd."""
import numpy as np
import pytest
import torch

import adjoint_torch as at
import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["a", "b"])
def test_prune_matches_reference_order(mg, golden, case):
    g = golden("basis_prune")
    G = g["gamma_" + case]
    fail = g["fail_a"] if case == "a" else ()
    with mg.Context(0) as c:
        order, lam = c.basis_prune(G, fail)
    assert np.array_equal(order, g["order_" + case])
    _, lam_orc = oracle.basis_prune(G, fail)
    assert np.all(np.abs(lam - lam_orc) <= 1e-12 + 1e-9 * np.abs(lam_orc))


def test_prune_device_gamma_and_edges(mg):
    q, tri, cl = mg.workload(120, 5)
    with mg.Context(0) as c:
        c.set_basis(2, 120, q)
        c.set_modes(tri)
        G = c.gamma()
        o1, l1 = c.basis_prune(None, [0, 34])
        o2, l2 = c.basis_prune(G, [0, 34])
        assert np.array_equal(o1, o2) and np.array_equal(l1, l2)
        assert sorted(o1.tolist()) == list(range(1, 34))
        # one and two active modes
        o, l = c.basis_prune(G[:2, :2], [1])
        assert o.tolist() == [0] and l.tolist() == [1.0]
        o, l = c.basis_prune(G[:2, :2])
        assert o.tolist() == [0, 1] and l[1] == 1.0
        with pytest.raises(mg.ModalError):
            c.basis_prune(G, [3, 3])
        with pytest.raises(mg.ModalError):
            c.basis_prune(G, [35])


def test_prune_bspline_workload_first_steps(mg):
    """364 modes of the 64-B-spline basis (lmax 1000): the GPU order's first
    three removals and their lambda against the numpy restatement."""
    C, Bw, tri, cl = mg.bspline_workload(1000, 12, 64, seed=4)
    with mg.Context(0) as c:
        c.set_basis(2, 1000, Bw @ C.T)
        c.set_modes(tri)
        G = c.gamma()
        c.profile(True)
        order, lam = c.basis_prune()
        ms, _ = c.timer("prune")
    print(f"prune 364 modes: {ms:.1f} ms")
    assert sorted(order.tolist()) == list(range(364))
    o_ref, l_ref = oracle.basis_prune(G, steps=3)
    assert np.array_equal(order[:3], o_ref)
    assert np.all(np.abs(lam[:3] - l_ref) <= 1e-12 + 1e-9 * np.abs(l_ref))
    # lambda_min never decreases along the greedy path (interlacing)
    assert np.all(np.diff(lam[:-1]) >= -1e-12)


def test_lambda_min_gradient_matches_torch(mg):
    lmax, P = 120, 4
    cl = mg.synthetic_cl(lmax)
    q = mg.weighted_q(mg.legendre_q(2, lmax, P), cl, 2)
    tri = mg.mode_triples(P)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tri)
        c.init_glint()
        mu, w = c.get_gl()
        c.gamma(download=False)
        lam, v, dq = c.lambda_min(grad=True)
    pr = at.Problem(mu, w, 2, lmax, tri, cl, None)
    qt = torch.tensor(q, requires_grad=True)
    G = pr.gamma(qt)
    d = torch.sqrt(torch.diagonal(G))
    lam_ref = torch.linalg.eigvalsh(G / torch.outer(d, d))[0]
    lam_ref.backward()
    assert abs(lam - lam_ref.item()) <= 1e-12 + 1e-9 * abs(lam_ref.item())
    g = qt.grad.numpy()
    assert np.linalg.norm(dq - g) / np.linalg.norm(g) <= 1e-7
