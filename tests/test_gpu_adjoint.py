"""GPU adjoint: gradients of Gamma, alpha and the projection-residual objective
with respect to the basis values q[L][P], from the library's hand-written
kernels, against torch float64 autograd of the same forward quantities
(tests/adjoint_torch.py) and central finite differences.  The library is
wrapped in a torch.autograd.Function here, in the tests only."""
import numpy as np
import pytest
import torch
from conftest import rel_fro

import adjoint_torch as at

pytestmark = pytest.mark.gpu

LMIN = 2


def _ctx(mg, lmax, q, tri, cl, mu=None, w=None):
    c = mg.Context(0)
    c.set_basis(LMIN, lmax, q)
    c.set_modes(tri)
    c.set_spectrum(cl)
    if mu is not None:
        c.set_gl(mu, w)
    c.init_glint()
    return c


def _small(mg, lmax=120, P=5):
    cl = mg.synthetic_cl(lmax)
    qraw = mg.legendre_q(LMIN, lmax, P)
    return cl, qraw, mg.weighted_q(qraw, cl, LMIN), mg.mode_triples(P)


def test_project_gl_modes_as_shapes(mg):
    lmax, P = 120, 5
    cl, qraw, q, tri = _small(mg, lmax, P)
    idx = [0, 4, 11, len(tri) - 1]
    shapes = []
    for m in idx:
        tab = np.zeros((1, 3, lmax + 1))
        for a in range(3):
            tab[0, a, LMIN:] = qraw[:, tri[m][a]]
        shapes.append({"kind": mg.SHAPE_SEPARABLE, "tab": tab})
    with _ctx(mg, lmax, q, tri, cl) as c:
        G = c.gamma()
        beta, n2 = c.project_gl(shapes)
        assert rel_fro(beta, G[idx]) <= 1e-12
        assert np.max(np.abs(n2 - G[idx, idx]) / G[idx, idx]) <= 1e-12
        c.orthogonalise()
        J, _ = c.adjoint_residual(shapes, grad=False)
        assert abs(J) <= 1e-10


def test_gamma_vjp_matches_torch(mg):
    lmax, P = 120, 5
    cl, qraw, q, tri = _small(mg, lmax, P)
    with _ctx(mg, lmax, q, tri, cl) as c:
        mu, w = c.get_gl()
        N = len(tri)
        Gup = np.random.default_rng(3).standard_normal((N, N))
        dq = c.gamma_vjp(Gup)
    pr = at.Problem(mu, w, LMIN, lmax, tri, cl, None)
    qt = torch.tensor(q, requires_grad=True)
    (pr.gamma(qt) * torch.tensor(Gup)).sum().backward()
    assert rel_fro(dq, qt.grad.numpy()) <= 1e-11


def test_project_gl_and_vjp_match_torch(mg):
    lmax, P = 120, 5
    cl, qraw, q, tri = _small(mg, lmax, P)
    shapes = mg.separable_shapes(lmax, 5, 11, 1, 3)
    with _ctx(mg, lmax, q, tri, cl) as c:
        mu, w = c.get_gl()
        beta, n2 = c.project_gl(shapes)
        up = np.random.default_rng(5).standard_normal(beta.shape)
        dq = c.project_gl_vjp(shapes, up)
    pr = at.Problem(mu, w, LMIN, lmax, tri, cl, shapes)
    qt = torch.tensor(q, requires_grad=True)
    b_ref, n2_ref = pr.beta_norm2(qt)
    assert rel_fro(beta, b_ref.detach().numpy()) <= 1e-12
    assert np.max(np.abs(n2 - n2_ref.detach().numpy()) / n2_ref.detach().numpy()) <= 1e-12
    (b_ref * torch.tensor(up)).sum().backward()
    assert rel_fro(dq, qt.grad.numpy()) <= 1e-11


def test_alpha_gl_vjp_matches_torch(mg):
    lmax, P = 120, 4   # 20 modes: Cholesky branch
    cl, qraw, q, tri = _small(mg, lmax, P)
    shapes = mg.separable_shapes(lmax, 4, 13, 1, 2)
    with _ctx(mg, lmax, q, tri, cl) as c:
        mu, w = c.get_gl()
        c.gamma()
        _, _, branch, _ = c.orthogonalise()
        assert branch == 0
        up = np.random.default_rng(9).standard_normal((len(shapes), len(tri)))
        alpha, dq = c.alpha_gl(shapes, up)
    pr = at.Problem(mu, w, LMIN, lmax, tri, cl, shapes)
    qt = torch.tensor(q, requires_grad=True)
    a_ref = pr.alpha(qt)
    assert rel_fro(alpha, a_ref.detach().numpy()) <= 1e-8
    (a_ref * torch.tensor(up)).sum().backward()
    assert rel_fro(dq, qt.grad.numpy()) <= 1e-7


class _Cfg4Residual(torch.autograd.Function):
    """J(C): the library's forward (FP64 Gamma, Cholesky, GL projection) and
    its adjoint, with the chain rule to the B-spline coefficients C[P][nb]:
    q~ = Bw C^T, dJ/dC = (dJ/dq~)^T Bw."""

    @staticmethod
    def forward(fctx, C, run):
        J, dq = run(C.detach().cpu().numpy(), True)
        fctx.save_for_backward(torch.from_numpy(dq.T @ run.Bw))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(fctx, gout):
        (dC,) = fctx.saved_tensors
        return gout * dC, None


class _Runner:
    def __init__(self, mg, c, Bw, shapes):
        self.c, self.Bw, self.shapes = c, Bw, shapes
        self.branches = []

    def __call__(self, C, grad):
        c = self.c
        c.set_basis(LMIN, 1000, self.Bw @ C.T)
        c.init_glint()
        c.gamma(download=False)
        _, _, br, _ = c.orthogonalise(download=False)
        self.branches.append(br)
        return c.adjoint_residual(self.shapes, grad=grad)


def test_cfg4_objective_gradient(mg):
    """lmax 1000, 12 functions of 64 cubic B-splines (364 modes), n_mu 1501,
    32 seeded shapes: the gradient with respect to the 12 x 64 coefficients
    against the torch float64 reference gradient and central differences
    (h = 1e-6)."""
    C0, Bw, tri, cl = mg.bspline_workload(1000, 12, 64, seed=4)
    shapes = mg.separable_shapes(1000, 32, 40, 1, 2)
    with mg.Context(0) as c:
        c.set_basis(LMIN, 1000, Bw @ C0.T)
        c.set_modes(tri)
        c.set_spectrum(cl)
        c.init_glint()
        mu, w = c.get_gl()
        assert mu.size == 1501
        run = _Runner(mg, c, Bw, shapes)
        C = torch.tensor(C0, requires_grad=True)
        J = _Cfg4Residual.apply(C, run)
        J.backward()
        grad = C.grad.numpy().copy()
        assert run.branches[-1] == 0
        # central finite differences along random directions and single coefficients
        rng = np.random.default_rng(17)
        h = 1e-6
        dirs = [rng.standard_normal(C0.shape) for _ in range(3)]
        for (p, j) in [(0, 0), (5, 31), (11, 63)]:
            e = np.zeros_like(C0)
            e[p, j] = 1.0
            dirs.append(e)
        for d in dirs:
            jp, _ = run(C0 + h * d, False)
            jm, _ = run(C0 - h * d, False)
            fd = (jp - jm) / (2 * h)
            an = float(np.sum(grad * d))
            assert abs(fd - an) <= 2e-6 * max(abs(an), 1e-3 * np.abs(grad).max() * np.abs(d).sum()), (fd, an)
    # torch float64 autograd of the same objective (on the GPU when available)
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    pr = at.Problem(mu, w, LMIN, 1000, tri, cl, shapes, device=dev)
    Ct = torch.tensor(C0, device=dev, requires_grad=True)
    Jr = pr.objective(torch.tensor(Bw, device=dev) @ Ct.T)
    Jr.backward()
    assert abs(J.item() - Jr.item()) <= 1e-11 * abs(Jr.item())
    assert rel_fro(grad, Ct.grad.cpu().numpy()) <= 1e-9
