"""The CPU oracle pinned against golden vectors produced by the reference's own
sources compiled in place (tests/golden/make_golden.py), and against
mathematical known answers."""
import numpy as np
import pytest
from conftest import rel_fro, rel_max


@pytest.mark.parametrize("n", [751, 1501, 3001])
def test_gl_nodes_match_reference_asy(orc, golden, n):
    g = golden("gl_asy")
    x, w = orc.gl_nodes(n)
    assert np.max(np.abs(x - g[f"x{n}"])) <= 2e-16
    assert np.max(np.abs(w - g[f"w{n}"]) / g[f"w{n}"]) <= 5e-15


def test_gl_reference_asy_is_approximate_at_small_n(orc, golden):
    # asy() uses large-n asymptotic expansions; at n = 31 its weights are off
    # by ~2e-10 and its rule no longer integrates x^60 exactly.  The oracle is.
    g = golden("gl_asy")
    x, w = orc.gl_nodes(31)
    assert np.max(np.abs(w - g["w31"]) / w) < 1e-9
    exact = 2.0 / 61.0
    assert abs(np.sum(w * x ** 60) - exact) / exact < 1e-13
    assert abs(np.sum(g["w31"] * g["x31"] ** 60) - exact) / exact > 1e-12


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 31, 91, 751])
def test_gl_nodes_exactness(orc, n):
    x, w = orc.gl_nodes(n)
    assert np.all(np.diff(x) > 0)
    assert np.allclose(x, -x[::-1], atol=0, rtol=0) or np.max(np.abs(x + x[::-1])) < 1e-16
    for m in range(0, n):  # exact for degree <= 2n-1
        exact = 2.0 / (2 * m + 1)
        assert abs(np.sum(w * x ** (2 * m)) - exact) <= 1e-13 * exact + 1e-16


def test_legendre_table_matches_scipy(orc):
    from scipy.special import eval_legendre
    mu = np.linspace(-1, 1, 41)
    t = orc.legendre_table(mu, 300)
    l = np.arange(301)
    ref = (2 * l + 1) ** (2 / 3) * eval_legendre(l[None, :], mu[:, None])
    assert np.max(np.abs(t - ref)) / np.max(np.abs(ref)) < 1e-12


def test_basis_legendre_matches_reference(orc, golden):
    g = golden("basis_legendre")
    b = orc.basis_legendre(g["values"], 9, 2.0, 500.0)
    assert np.max(np.abs(b - g["basis"])) <= 1e-14


def test_geometric_matches_reference(orc, golden):
    g = golden("geometric")
    v = np.array([orc.geometric(int(a), int(b), int(c)) for a, b, c in g["pts"]])
    nz = g["geo"] != 0
    assert np.array_equal(v == 0, g["geo"] == 0)
    assert np.max(np.abs(v[nz] - g["geo"][nz]) / g["geo"][nz]) < 1e-14


def _walk(orc, lmin, lmax, n):
    import ctypes
    i, j, k = ctypes.c_int(lmin), ctypes.c_int(lmin), ctypes.c_int(lmin)
    # start as check_ijk_min_XXX: (lmin, lmin, lmin + parity)
    if (3 * lmin) % 2 == 1:
        k.value += 1
    pts = []
    for _ in range(n):
        pts.append((i.value, j.value, k.value))
        if not orc.L.orc_tetrapyd_next(lmax, ctypes.byref(i), ctypes.byref(j), ctypes.byref(k)):
            pts.append((i.value, j.value, k.value))
            break
    return np.array(pts[:n])


def test_tetrapyd_walk_and_counts(orc, golden):
    g = golden("tetrapyd")
    w = _walk(orc, 2, 30, 400)
    assert np.array_equal(w, g["walk"][:len(w)])
    for key in g.files:
        if key.startswith("count_"):
            a, b = map(int, key[6:].split("_"))
            assert orc.tetrapyd_count(a, b) == int(g[key])


def test_tetrapyd_walk_is_the_even_triangle_set(orc):
    lmin, lmax = 3, 40
    n = orc.tetrapyd_count(lmin, lmax)
    w = _walk(orc, lmin, lmax, n)
    enum = {(i, j, k) for i in range(lmin, lmax + 1) for j in range(i, lmax + 1)
            for k in range(j, min(i + j, lmax) + 1) if (i + j + k) % 2 == 0}
    assert len(w) == n == len(enum)
    assert set(map(tuple, w.tolist())) == enum


@pytest.mark.parametrize("name", ["small", "cfg1"])
def test_gamma_matches_reference(orc, golden, mg, name):
    g = golden("gamma_" + name)
    gl = golden("gl_asy")
    lmax, P = int(g["lmax"]), int(g["P"])
    q, tr, cl = mg.workload(lmax, P)
    nmu = 3 * lmax // 2 + 1
    x, w = gl[f"x{nmu}"], gl[f"w{nmu}"]
    M = orc.mij(orc.legendre_table(x, lmax), 2, lmax, q)
    G = orc.gamma(M, w, tr)
    assert rel_fro(G, g["gamma"]) <= 1e-13
    assert rel_max(G, g["gamma"]) <= 1e-13
    assert np.array_equal(G, G.T)


def test_projection_matches_reference_small(orc, golden, mg):
    g = golden("gamma_small")
    lmax, P, S = int(g["lmax"]), int(g["P"]), int(g["S"])
    q, tr, cl = mg.workload(lmax, P)
    shapes = mg.separable_shapes(lmax, S // 2, seed=0) + mg.bump_shapes(S - S // 2, seed=1)
    for s, sh in enumerate(shapes):
        b = orc.project(2, lmax, q, tr, cl, sh, nthreads=4)
        assert rel_fro(b, g["beta"][s]) <= 1e-13


def test_cholesky_restatement_against_lapack(orc):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((50, 50))
    G = A @ A.T + 50 * np.eye(50)
    o, lam, fail = orc.ortho_cholesky(G)
    assert fail == -1
    norm = np.sqrt(np.diag(G))
    Lref = np.linalg.cholesky(G / np.outer(norm, norm))
    assert np.allclose(o, norm[:, None] * Lref, rtol=1e-12, atol=1e-12)
    assert np.allclose(o @ o.T, G, rtol=1e-12)
    assert np.allclose(lam @ o, np.eye(50), atol=1e-12)
    assert np.array_equal(np.triu(lam, 1), np.zeros((50, 50)))


def test_cholesky_restatement_reports_failing_pivot(orc):
    G = np.eye(6)
    G[3, 3] = -1.0
    G[3, 3] = 1.0
    G[2, 4] = G[4, 2] = 2.0  # minor [[1,2],[2,1]] is indefinite
    _, _, fail = orc.ortho_cholesky(G)
    assert fail == 4


def test_pca_restatement_properties():
    import oracle
    rng = np.random.default_rng(4)
    A = rng.standard_normal((30, 12))
    G = A @ A.T + 1e-3 * np.eye(30)
    inv, lam, r = oracle.ortho_pca(G)
    assert r == 30
    assert np.allclose(lam @ G @ lam.T, np.eye(30), atol=1e-8)
    assert np.allclose(inv @ inv.T, G, rtol=1e-10, atol=1e-10)
    G2 = A @ A.T  # rank 12: some eigenvalues come out <= 0 in FP64
    inv2, lam2, r2 = oracle.ortho_pca(G2)
    assert 12 <= r2 <= 30
    assert np.all(lam2[r2:] == 0) and np.all(inv2[:, r2:] == 0)


def test_alpha_restatement(orc):
    rng = np.random.default_rng(5)
    A = rng.standard_normal((40, 40))
    G = A @ A.T + 40 * np.eye(40)
    o, lam, _ = orc.ortho_cholesky(G)
    beta = rng.standard_normal(40)
    a, mR = orc.alpha(o, lam, beta)
    assert np.allclose(a, np.linalg.solve(G, beta), rtol=1e-10)
    assert np.allclose(mR, lam @ beta, rtol=1e-10, atol=1e-12)


def test_dense_form_matches_reference(orc, golden, mg):
    """modify_bispectrum + calculate_modes (calculate_modes.c:6-79) vs the in-place reference."""
    import numpy as np
    g = golden("modes_dense")
    lmax, P = int(g["lmax"]), int(g["P"])
    size = g["modified"].shape[0]
    q, tr, cl = mg.workload(lmax, P)
    l = np.arange(size, dtype=np.float64)
    l[0] = 1.0
    raw = np.einsum("i,j,k->ijk", l ** -1.2, l ** -0.7, l ** -1.5)
    raw = (raw + raw.transpose(1, 2, 0) + raw.transpose(2, 0, 1)) / 3.0
    mod = orc.modify_bispectrum(raw, np.arange(size), cl)
    nz = g["modified"] != 0
    assert np.array_equal(mod != 0, nz)
    assert np.max(np.abs(mod[nz] - g["modified"][nz]) / np.abs(g["modified"][nz])) <= 1e-14
    beta = orc.calculate_modes(2, lmax, q, tr, g["modified"])
    assert rel_fro(beta, g["beta"]) <= 1e-13


def _transfer_inputs(lmax, Pp, xsize):
    import numpy as np
    xvec = np.linspace(1000.0, 12000.0, xsize)
    l = np.arange(lmax + 1.0)
    qt = np.zeros((xsize, Pp, lmax + 1))
    for xi, x in enumerate(xvec):
        for p in range(Pp):
            qt[xi, p] = np.cos((p + 1) * x / 4000.0) * np.sin(0.1 * l * (1 + p) + x / 3000.0) / (1.0 + l)
    return xvec, qt


@pytest.mark.parametrize("name", ["a", "b"])
def test_gamma_3d_matches_reference(orc, golden, mg, name):
    """calculate_gamma_TTT_3D_nested (the rflag_do3D == 0 path of gamma_mpi.c) vs the
    in-place reference: the tetrapyd sum with the radial trapezium integrals."""
    g = golden("gamma_3d")
    lmax, P, Pp, xsize = (int(v) for v in g["dims_" + name])
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = mg.transfer_workload(lmax, Pp, xsize)
    G = orc.gamma_3d(2, lmax, q, tr, cl, xvec, qt, mg.mode_triples(Pp), float(g["dphi_" + name][0]))
    assert rel_max(G, g["gamma_" + name]) <= 1e-13


@pytest.mark.parametrize("name", ["a", "b"])
def test_transfer_gamma_matches_reference(orc, golden, mg, name):
    """calculate_gamma_2d path of calculate_gamma.c vs the in-place reference."""
    g = golden("gamma_transfer")
    lmax, P, Pp, xsize = (int(v) for v in g["dims_" + name])
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = _transfer_inputs(lmax, Pp, xsize)
    x, w = golden("gl_asy")["x91"], golden("gl_asy")["w91"]
    nmu = 3 * lmax // 2 + 1
    if nmu != 91:
        x, w = orc.gl_nodes(nmu)
    G = orc.gamma_transfer(2, lmax, q, tr, cl, x, w, xvec, qt, mg.mode_triples(Pp), 0.7)
    tol = 1e-14 if nmu == 91 else 1e-12  # own nodes vs asy() at n = 136
    assert rel_max(G, g["gamma_" + name]) <= tol


def test_cubic_spline_integral_exact_for_cubics(orc):
    import numpy as np
    x = np.sort(np.random.default_rng(2).uniform(0, 3, 25))
    y = 2 - x + 0.5 * x ** 2 - 0.25 * x ** 3
    exact = lambda t: 2 * t - t ** 2 / 2 + t ** 3 / 6 - t ** 4 / 16  # noqa: E731
    assert abs(orc.integrate_cubic_spline(x, y) - (exact(x[-1]) - exact(x[0]))) < 1e-12


@pytest.mark.parametrize("case", ["a", "b"])
def test_basis_prune_matches_reference_driver(golden, case):
    # basis_optimisation_mpi.c's own main() (in place, Jacobi stand-in for dsyevr)
    import oracle
    g = golden("basis_prune")
    fail = g["fail_a"] if case == "a" else ()
    order, lam = oracle.basis_prune(g["gamma_" + case], fail)
    assert np.array_equal(order, g["order_" + case])
    # the reference prints lambda with %e (7 significant digits)
    assert np.max(np.abs(lam - g["lam_" + case]) / np.abs(lam)) <= 6e-7


def test_polarised_gamma_oracle_vs_reference(orc, golden):
    # calculate_orthol with do_polarisation: TTT, TTE, TEE, EEE (the reference in place)
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import pol_inputs
    g = golden("gamma_pol")
    lmaxT, lmaxE, lminE = (int(v) for v in g["dims"])
    cl, qT, qE, ttt, tte, tee, eee = pol_inputs(lmaxT, lmaxE, lminE)
    pl = orc.legendre_table(g["nodes"], max(lmaxT, lmaxE))
    MT = orc.mij(np.ascontiguousarray(pl[:, :lmaxT + 1]), 2, lmaxT, qT)
    ME = orc.mij(pl, lminE, lmaxE, qE)
    gT = orc.gamma(MT, g["weights"], ttt)
    g1, g2, g3 = orc.gamma_pol(MT, ME, g["weights"], tte, tee, eee)
    for got, want in zip((gT, g1, g2, g3), g["gamma"]):
        assert rel_max(got, want) <= 1e-14


def test_polarised_transfer_oracle_vs_reference(orc, golden):
    # calculate_gamma_2d with do_polarisation (E weights, calculate_gamma.c:142-183)
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import pol_transfer_inputs
    g = golden("gamma_transfer_pol")
    d = pol_transfer_inputs()
    out = orc.gamma_transfer_pol(2, d["lmax"], d["qT"], d["lminE"], d["lmaxE"], d["qE"], d["tte"], d["tee"], d["eee"],
                                 d["spec9"], d["fsky_t"], d["fsky_e"], g["nodes"], g["weights"], d["xvec"], d["qtT"],
                                 d["qtE"], d["prim"], d["dphi"])
    for f in range(3):
        assert rel_max(out[f], g["gamma"][f + 1]) <= 1e-14


def _prim_inputs(kmax_i):
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import prim_inputs
    return prim_inputs(kmax_i)


@pytest.mark.parametrize("name", ["a", "b"])
def test_prim_oracle_vs_reference(orc, golden, name):
    # calculate_ortho / calculate_eigen / integrate_template2 (the reference in place)
    g = golden("prim")
    kmin, kmax_i, kmax = g["grid_" + name]
    kmin, kmax_i = int(kmin), int(kmax_i)
    basis, prim, shapes = _prim_inputs(kmax_i)
    assert rel_max(orc.prim_ortho(kmin, kmax_i, kmax, basis, prim), g["ortho_" + name]) <= 1e-15
    for n, sh in enumerate(shapes):
        a, n2 = orc.prim_eigen(kmin, kmax_i, kmax, basis, prim, sh)
        assert rel_max(a, g[f"alpha_{name}{n}"]) <= 1e-14
        assert abs(n2 - g[f"norm2_{name}{n}"][0]) <= 1e-14 * abs(n2)


def test_prim_walk_closed_form(orc):
    # the walk of get_ijk_next_prim covers min <= i < max, i <= j <= max,
    # j <= k <= min(max, i+j+2), then the end point (max, max, max)
    for kmin, kmax_i in [(1, 12), (0, 9), (3, 20), (2, 3)]:
        walk = orc.prim_walk(kmin, kmax_i)
        pts = [(i, j, k) for i in range(kmin, kmax_i) for j in range(i, kmax_i + 1)
               for k in range(j, min(kmax_i, i + j + 2) + 1)] + [(kmax_i,) * 3]
        assert [tuple(p) for p in walk] == pts
