"""GPU parity of the library's own FP64 symmetric eigensolver (modal_eigh; the
PCA branch of modal_orthogonalise and modal_basis_prune run on it) against
LAPACK through numpy.linalg.eigh, the stand-in for gsl_eigen_symmv
(ortho_late_mpi.c:775-776) and LAPACKE_dsyevr (basis_optimisation_mpi.c:279).
Tolerances, with eps = 2^-52 and ||A|| the spectral norm:
  eigenvalues      |w - w_lapack| <= 8 n eps ||A||
  residual         ||A V^T - V^T diag(w)||_F <= 8 n eps ||A||
  orthogonality    max |V V^T - I| <= 8 n eps"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = np.finfo(float).eps


@pytest.fixture(scope="module")
def ctx(mg):
    c = mg.Context(0)
    yield c
    c.close()


def check(ctx, A, vectors=True):
    n = A.shape[0]
    w, V = ctx.eigh(A, vectors)
    wr = np.linalg.eigvalsh(A)
    nrm = max(np.max(np.abs(wr)), 1e-300)
    tol = 8 * max(n, 4) * EPS * nrm
    assert np.all(np.diff(w) >= 0), "eigenvalues not ascending"
    assert np.max(np.abs(w - wr)) <= tol
    if vectors:
        res = np.linalg.norm(A @ V.T - V.T * w[None, :])
        assert res <= tol * max(1.0, np.sqrt(n) / 4)
        assert np.max(np.abs(V @ V.T - np.eye(n))) <= 8 * max(n, 4) * EPS
    return w, V


@pytest.mark.parametrize("n", [1, 2, 3, 5, 31, 32, 33, 64, 65, 97, 256, 513])
def test_eigh_random(ctx, n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, n))
    check(ctx, (X + X.T) / 2)


def test_eigh_values_only(ctx):
    rng = np.random.default_rng(7)
    X = rng.standard_normal((200, 200))
    w, V = check(ctx, X + X.T, vectors=False)
    assert V is None


@pytest.mark.parametrize("kind", ["zero", "identity", "repeated", "rank10", "graded", "wilkinson", "diagonal"])
def test_eigh_structured(ctx, kind):
    rng = np.random.default_rng(3)
    n = 300
    if kind == "zero":
        A = np.zeros((n, n))
    elif kind == "identity":
        A = np.eye(n)
    elif kind == "diagonal":
        A = np.diag(rng.standard_normal(n))
    elif kind == "repeated":  # three eigenvalues, each 100 times
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = (Q * np.repeat([-1.0, 0.5, 2.0], 100)[None, :]) @ Q.T
        A = (A + A.T) / 2
    elif kind == "rank10":
        X = rng.standard_normal((n, 10))
        A = X @ X.T
    elif kind == "graded":  # eigenvalues from 1 down to 1e-15, as a nearly dependent mode set gives
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = (Q * np.logspace(0, -15, n)[None, :]) @ Q.T
        A = (A + A.T) / 2
    else:  # Wilkinson W_{n}^+: pairs of nearly equal eigenvalues
        m = (n - 1) // 2
        A = np.diag(np.abs(np.arange(n) - m).astype(float)) + np.diag(np.ones(n - 1), 1) + np.diag(np.ones(n - 1), -1)
    if kind == "zero":
        w, V = ctx.eigh(A)
        assert np.all(w == 0) and np.max(np.abs(V @ V.T - np.eye(n))) <= 1e-14
        return
    check(ctx, A)


def test_eigh_normalised_gamma(ctx, mg):
    """The matrix the PCA branch sees: the normalised FP64 Gamma of l = 2..500, P = 10 (N = 220)."""
    q, tr, cl = mg.workload(500, 10)
    ctx.set_basis(2, 500, q)
    ctx.set_modes(tr)
    G = ctx.gamma(mg.PREC_FP64)
    nrm = np.sqrt(np.diag(G))
    check(ctx, G / np.outer(nrm, nrm))


@pytest.mark.parametrize("floor", [1e-10, 1e-6, 1e-4])
def test_pca_branch_against_numpy_with_floor(mg, floor):
    """PCA outputs of a nearly dependent Gamma (l = 2..600, P = 16, N = 816) with
    an eigenvalue floor: the same kept rank as numpy, the kept-subspace projector
    and alpha = lambda^T lambda beta equal to the numpy restatement."""
    import oracle
    lmax, P = 600, 16
    q, tr, cl = mg.workload(lmax, P)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        G = c.gamma(mg.PREC_FP64)
        c.set_pca_floor(floor)
        o, lam, branch, rank = c.orthogonalise(G, pca_flag=0)
        inv_ref, lam_ref, r_ref = oracle.ortho_pca(G, floor)
        assert branch == 1 and rank == r_ref
        nrm = np.sqrt(np.diag(G))
        e = np.linalg.eigvalsh(G / np.outer(nrm, nrm))[::-1]
        # projector onto the kept eigenvectors of the normalised Gamma
        U = (lam[:rank] * nrm[None, :] * np.sqrt(e[:rank])[:, None]).T
        Ur = (lam_ref[:rank] * nrm[None, :] * np.sqrt(e[:rank])[:, None]).T
        gap = e[rank - 1] - (e[rank] if rank < len(e) else 0.0)
        tol_p = max(1e-10, 64 * len(e) * EPS * e[0] / gap)
        assert np.max(np.abs(U @ U.T - Ur @ Ur.T)) <= tol_p
        beta = c.project(mg.separable_shapes(lmax, 2, seed=5))
        a, _ = c.alpha(2)
        a_ref = (lam_ref.T @ (lam_ref @ beta.T)).T
        assert np.max(np.abs(a - a_ref)) / np.max(np.abs(a_ref)) <= max(1e-8, tol_p * e[0] / e[rank - 1])
        c.set_pca_floor(0.0)
