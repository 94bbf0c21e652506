"""GPU parity of the plain FP64 form against the oracle and the golden vectors
of the reference (tolerances written per test).  Every call goes through the
C ABI of libmodal_gb300.so."""
import numpy as np
import pytest
from conftest import rel_fro, rel_max

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(mg):
    c = mg.Context(0)
    yield c
    c.close()


# ---------------------------------------------------------------- primitives

@pytest.mark.parametrize("n", [1, 2, 3, 31, 91, 751, 3001, 3751])
def test_gl_nodes_vs_oracle(mg, orc, n):
    x, w = mg.gl_nodes(n)
    xo, wo = orc.gl_nodes(n)
    assert np.max(np.abs(x - xo)) <= 5e-16
    assert np.max(np.abs(w - wo) / wo) <= 1e-13  # FP64 recurrence vs long double


@pytest.mark.parametrize("n", [751, 1501, 3001])
def test_gl_nodes_vs_reference_asy(mg, golden, n):
    g = golden("gl_asy")
    x, w = mg.gl_nodes(n)
    assert np.max(np.abs(x - g[f"x{n}"])) <= 5e-16
    assert np.max(np.abs(w - g[f"w{n}"]) / g[f"w{n}"]) <= 1e-13


def test_legendre_table_vs_oracle(mg, orc, golden):
    x = golden("gl_asy")["x751"]
    t = mg.legendre_table(x, 500)
    to = orc.legendre_table(x, 500)
    assert rel_max(t, to) <= 1e-13
    # edge nodes +-1 and 0 take the exact branches
    e = np.array([-1.0, 0.0, 1.0])
    assert np.max(np.abs(mg.legendre_table(e, 50) - orc.legendre_table(e, 50))) <= 1e-12


def test_basis_legendre_vs_reference(mg, golden):
    g = golden("basis_legendre")
    b = mg.basis_legendre(g["values"], 9, 2.0, 500.0)
    assert np.max(np.abs(b - g["basis"])) <= 1e-14


def test_geometric_vs_reference(mg, golden):
    g = golden("geometric")
    v = mg.geometric(g["pts"])
    nz = g["geo"] != 0
    assert np.array_equal(v == 0, g["geo"] == 0)
    assert np.max(np.abs(v[nz] - g["geo"][nz]) / g["geo"][nz]) <= 1e-14


# --------------------------------------------------------------------- Gamma

@pytest.mark.parametrize("name", ["small", "cfg1"])
def test_gamma_vs_reference_with_reference_nodes(mg, golden, ctx, name):
    """Bit-level parity target 1e-12: same inputs and the reference's own asy()
    nodes, Gamma vs calculate_orthol over all pairs."""
    g = golden("gamma_" + name)
    lmax, P = int(g["lmax"]), int(g["P"])
    q, tr, cl = mg.workload(lmax, P)
    nmu = 3 * lmax // 2 + 1
    gl = golden("gl_asy")
    ctx.set_basis(2, lmax, q)
    ctx.set_modes(tr)
    ctx.set_gl(gl[f"x{nmu}"], gl[f"w{nmu}"])
    G = ctx.gamma(mg.PREC_FP64)
    assert rel_fro(G, g["gamma"]) <= 1e-12
    assert rel_max(G, g["gamma"]) <= 1e-12
    assert np.array_equal(G, G.T)
    # per-pair interface (calculate_orthol)
    for m, n in [(0, 0), (1, 7), (len(tr) - 1, 3)]:
        assert abs(ctx.orthol_pair(m, n) - g["gamma"][m, n]) <= 1e-12 * np.abs(g["gamma"]).max()


def test_mij_vs_oracle(mg, orc, golden, ctx):
    lmax, P = 500, 10
    q, tr, cl = mg.workload(lmax, P)
    gl = golden("gl_asy")
    ctx.set_basis(2, lmax, q)
    ctx.set_modes(tr)
    ctx.set_gl(gl["x751"], gl["w751"])
    ctx.init_glint()
    M = ctx.get_mij()
    Mo = orc.mij(orc.legendre_table(gl["x751"], lmax), 2, lmax, q)
    assert M.shape == Mo.shape
    assert rel_max(M, Mo) <= 1e-12
    x, w = ctx.get_gl()
    assert np.array_equal(x, gl["x751"]) and np.array_equal(w, gl["w751"])


def test_gamma_own_nodes_vs_oracle(mg, orc, ctx):
    lmax, P = 300, 7
    q, tr, cl = mg.workload(lmax, P)
    ctx.set_basis(2, lmax, q)
    ctx.set_modes(tr)
    ctx2 = mg.Context(0)
    ctx2.set_basis(2, lmax, q)
    ctx2.set_modes(tr)
    G = ctx2.gamma(mg.PREC_FP64)
    ctx2.close()
    x, w = orc.gl_nodes(3 * lmax // 2 + 1)
    Go = orc.gamma(orc.mij(orc.legendre_table(x, lmax), 2, lmax, q), w, tr)
    assert rel_fro(G, Go) <= 1e-12


@pytest.mark.parametrize("P,modes", [(1, [[0, 0, 0]]), (3, [[2, 1, 0], [0, 0, 0], [1, 1, 1], [2, 1, 0]]),
                                     (5, None)])
def test_gamma_edge_cases(mg, orc, P, modes):
    """N = 1, unsorted and duplicated triples, N not a multiple of the tile."""
    lmax = 40
    q, tr, cl = mg.workload(lmax, P)
    tr = np.array(modes, dtype=np.int32) if modes is not None else tr
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        G = c.gamma(mg.PREC_FP64)
    x, w = orc.gl_nodes(3 * lmax // 2 + 1)
    Go = orc.gamma(orc.mij(orc.legendre_table(x, lmax), 2, lmax, q), w, tr)
    assert rel_max(G, Go) <= 1e-12


def test_bad_arguments_are_rejected(mg):
    with mg.Context(0) as c:
        with pytest.raises(mg.ModalError) as e:
            c.gamma()
        assert e.value.status == 6
        q, tr, cl = mg.workload(40, 3)
        c.set_basis(2, 40, q)
        with pytest.raises(mg.ModalError) as e:
            c.set_modes(np.array([[0, 1, 3]]))
        assert e.value.status == 1
        with pytest.raises(mg.ModalError):
            c.set_basis(2, 40, np.zeros((39, 65)))


# ---------------------------------------------------------- orthogonalisation

def _spd_gamma(mg, golden):
    g = golden("gamma_small")
    return g["gamma"]


def test_cholesky_branch_vs_oracle(mg, orc, golden):
    G = _spd_gamma(mg, golden)
    N = G.shape[0]
    o_ref, lam_ref, fail = orc.ortho_cholesky(G)
    assert fail == -1
    with mg.Context(0) as c:
        q, tr, cl = mg.workload(60, 4)
        c.set_basis(2, 60, q)
        c.set_modes(tr)
        o, lam, branch, rank = c.orthogonalise(G, pca_flag=1)
    assert branch == 0 and rank == N
    assert rel_max(o, o_ref) <= 1e-10
    assert rel_max(lam, lam_ref) <= 1e-8
    assert np.array_equal(np.triu(o, 1), np.zeros((N, N))) and np.array_equal(np.triu(lam, 1), np.zeros((N, N)))
    assert rel_max(o @ o.T, G) <= 1e-12  # backward error


def test_cholesky_blocked_large_spd(mg, orc):
    """Several 64-wide panels, N not a multiple of 64."""
    rng = np.random.default_rng(11)
    N = 301
    A = rng.standard_normal((N, N))
    G = A @ A.T + N * np.eye(N)
    o_ref, lam_ref, _ = orc.ortho_cholesky(G)
    with mg.Context(0) as c:
        q, _, _ = mg.workload(60, 13)
        c.set_basis(2, 60, q)
        c.set_modes(mg.mode_triples(13)[:N])
        o, lam, branch, rank = c.orthogonalise(G, pca_flag=1)
    assert branch == 0
    assert rel_max(o, o_ref) <= 1e-12
    assert rel_max(lam, lam_ref) <= 1e-11
    assert np.max(np.abs(lam @ o - np.eye(N))) <= 1e-11



@pytest.mark.parametrize("lmax,P", [(2000, 30), (2500, 40)])
def test_gamma_fp64_benchmark_sizes_vs_oracle_pairs(mg, orc, lmax, P):
    """The FP64 Gamma at the benchmark sizes (l <= 2000, P = 30, N = 4960; l <=
    2500, P = 40, N = 11480) against the oracle's restatement of
    calculate_orthol (orthogonalisation_late.c:239-336) on the same nodes, for
    2000 random (m, n) pairs: within 1e-12 of max |Gamma|."""
    q, tr, cl = mg.workload(lmax, P)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.init_glint()
        G = c.gamma(mg.PREC_FP64)
        x, w = c.get_gl()
    M = orc.mij(orc.legendre_table(x, lmax), 2, lmax, q)
    rng = np.random.default_rng(lmax)
    pairs = rng.integers(0, len(tr), (2000, 2))
    ref = np.array([orc.orthol_pair(M, w, tr, int(m), int(n)) for m, n in pairs])
    got = G[pairs[:, 0], pairs[:, 1]]
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(G))

def test_pca_branch_forced_and_on_failure(mg):
    import oracle
    rng = np.random.default_rng(12)
    N = 150
    A = rng.standard_normal((N, 40))
    G_def = A @ A.T  # rank 40: not positive definite
    with mg.Context(0) as c:
        q, _, _ = mg.workload(60, 10)
        c.set_basis(2, 60, q)
        c.set_modes(mg.mode_triples(10)[:N])
        for G, flag in [(A @ A.T + np.eye(N), 0), (G_def, 1)]:
            o, lam, branch, rank = c.orthogonalise(G, pca_flag=flag)
            inv_ref, lam_ref, r_ref = oracle.ortho_pca(G)
            assert branch == 1
            if flag == 0:
                assert rank == r_ref == N
            else:  # 40 true positive eigenvalues, the rest at round-off level with either sign
                assert rank >= 40 and r_ref >= 40
            r = min(rank, r_ref, 40 if flag == 1 else N)
            # rows of lambda equal up to the sign of each eigenvector (well separated part)
            for i in range(min(r, 30)):
                s = np.sign(np.dot(lam[i], lam_ref[i]))
                assert np.max(np.abs(lam[i] - s * lam_ref[i])) <= 1e-8 * np.max(np.abs(lam_ref[i]))
            assert np.all(lam[rank:] == 0) and np.all(o[:, rank:] == 0)
        # eigenvalue floor: rank 40 exactly once the round-off eigenvalues are cut
        n = np.sqrt(np.diag(G_def))
        e = np.linalg.eigvalsh(G_def / np.outer(n, n))
        c.set_pca_floor(1e-10)
        _, lam, branch, rank = c.orthogonalise(G_def, pca_flag=1)
        assert branch == 1 and rank == int(np.sum(e > 1e-10 * e[-1])) == 40
        assert np.all(lam[40:] == 0)
        c.set_pca_floor(0.0)
        with pytest.raises(mg.ModalError):
            c.set_pca_floor(1.0)


# ---------------------------------------------------------------- projection

@pytest.mark.parametrize("name", ["small", "cfg1"])
def test_projection_vs_reference(mg, golden, name):
    g = golden("gamma_" + name)
    lmax, P, S = int(g["lmax"]), int(g["P"]), int(g["S"])
    q, tr, cl = mg.workload(lmax, P)
    shapes = mg.separable_shapes(lmax, S // 2, seed=0) + mg.bump_shapes(S - S // 2, seed=1)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        beta = c.project(shapes, mg.PREC_FP64)
        for s in range(S):
            assert rel_fro(beta[s], g["beta"][s]) <= 1e-12
        # one shape at a time gives the same as the batch
        b1 = c.project(shapes[1:2], mg.PREC_FP64)
        assert rel_fro(b1[0], beta[1]) <= 1e-14


@pytest.mark.parametrize("lmin,lmax,P", [(2, 3, 2), (2, 33, 3), (5, 64, 4), (7, 40, 1)])
def test_projection_edge_sizes_vs_oracle(mg, orc, lmin, lmax, P):
    cl = mg.synthetic_cl(lmax)
    q = mg.weighted_q(mg.legendre_q(lmin, lmax, P), cl, lmin)
    tr = mg.mode_triples(P)
    shapes = mg.separable_shapes(lmax, 1, seed=3) + mg.bump_shapes(1, seed=4)
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        beta = c.project(shapes)
    for s, sh in enumerate(shapes):
        bo = orc.project(lmin, lmax, q, tr, cl, sh, nthreads=2)
        assert rel_fro(beta[s], bo) <= 1e-12


def test_projection_term_counts_vs_oracle(mg, orc):
    """FP64 separable shapes at the row-coefficient boundary: 1, 8 (row
    coefficients) and 9 terms (the six-ordering sum) against the oracle, 1e-12,
    in one call with a bump; odd l_max and l_min > 2."""
    lmin, lmax, P = 3, 71, 5
    cl = mg.synthetic_cl(lmax)
    q = mg.weighted_q(mg.legendre_q(lmin, lmax, P), cl, lmin)
    tr = mg.mode_triples(P)
    shapes = (mg.separable_shapes(lmax, 1, seed=31, tmin=1, tmax=1) + mg.separable_shapes(lmax, 1, seed=32, tmin=8, tmax=8)
              + mg.separable_shapes(lmax, 1, seed=33, tmin=9, tmax=9) + mg.bump_shapes(1, seed=34))
    assert [sh["tab"].shape[0] for sh in shapes[:3]] == [1, 8, 9]
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        beta = c.project(shapes)
    for s, sh in enumerate(shapes):
        assert rel_fro(beta[s], orc.project(lmin, lmax, q, tr, cl, sh, nthreads=2)) <= 1e-12, s


# --------------------------------------------------------------------- alpha

def test_alpha_vs_oracle(mg, orc, golden):
    g = golden("gamma_small")
    G, beta = g["gamma"], g["beta"]
    o_ref, lam_ref, _ = orc.ortho_cholesky(G)
    with mg.Context(0) as c:
        q, tr, cl = mg.workload(60, 4)
        c.set_basis(2, 60, q)
        c.set_modes(tr)
        c.orthogonalise(G, pca_flag=1, download=False)
        a, mR = c.alpha(beta.shape[0], beta)
    for s in range(beta.shape[0]):
        a_ref, m_ref = orc.alpha(o_ref, lam_ref, beta[s])
        assert rel_fro(a[s], a_ref) <= 1e-8
        assert rel_fro(mR[s], m_ref) <= 1e-8
        # gamma-norm error of the reconstruction
        d = a[s] - a_ref
        assert np.sqrt(abs(d @ G @ d)) <= 1e-8 * np.sqrt(a_ref @ G @ a_ref)


@pytest.mark.parametrize("S", [1, 16, 17, 32, 40, 130])
def test_alpha_products_any_shape_count(mg, S):
    """alpha = (beta lambda^T) lambda and modesR = alpha orthol for S shapes: one
    or two 16-row passes of the skinny products (S <= 32) or the FP64-accurate
    tensor-core product (S > 32), against numpy on the downloaded
    orthogonalisation outputs."""
    rng = np.random.default_rng(40 + S)
    N = 200
    A = rng.standard_normal((N, N))
    G = A @ A.T + N * np.eye(N)
    beta = rng.standard_normal((S, N))
    with mg.Context(0) as c:
        q, _, _ = mg.workload(60, 12)
        c.set_basis(2, 60, q)
        c.set_modes(mg.mode_triples(12)[:N])
        o, lam, branch, rank = c.orthogonalise(G, pca_flag=1)
        a, mR = c.alpha(S, beta)
        a2, mR2 = c.alpha(S, beta)
    assert branch == 0 and rank == N
    a_ref = (beta @ lam.T) @ lam
    assert rel_fro(a, a_ref) <= 1e-12
    assert rel_fro(mR, a_ref @ o) <= 1e-12
    assert np.array_equal(a, a2) and np.array_equal(mR, mR2)  # fixed reduction order


@pytest.mark.parametrize("S", [3, 40])
def test_alpha_modesR_pca_branch_lower_triangle(mg, orc, S):
    """On the PCA branch orthol is dense; eigenmodetoday_mpi.c builds lambdainv
    from its lower triangle only, so modesR = alpha tril(orthol).  GPU alpha and
    modesR against the oracle's restatement on the downloaded outputs: 1e-12."""
    rng = np.random.default_rng(77)
    N = 180
    A = rng.standard_normal((N, N))
    G = A @ A.T + N * np.eye(N)
    beta = rng.standard_normal((S, N))
    with mg.Context(0) as c:
        q, _, _ = mg.workload(60, 12)
        c.set_basis(2, 60, q)
        c.set_modes(mg.mode_triples(12)[:N])
        o, lam, branch, rank = c.orthogonalise(G, pca_flag=0)
        a, mR = c.alpha(S, beta)
    assert branch == 1 and rank == N
    assert np.count_nonzero(np.triu(o, 1)) > 0  # dense: the truncation matters
    for s in range(S):
        a_o, m_o = orc.alpha(o, lam, beta[s])
        assert rel_max(a[s], a_o) <= 1e-12
        assert rel_max(mR[s], m_o) <= 1e-12
        assert rel_max(mR[s], a[s] @ np.tril(o)) <= 1e-12


def test_full_pipeline_on_device(mg, golden):
    """Gamma -> orthogonalise -> project -> alpha with everything left on the device."""
    g = golden("gamma_small")
    lmax, P, S = 60, 4, 4
    q, tr, cl = mg.workload(lmax, P)
    shapes = mg.separable_shapes(lmax, 2, seed=0) + mg.bump_shapes(2, seed=1)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        gl = golden("gl_asy")
        c.set_gl(gl["x91"], gl["w91"])
        c.gamma(mg.PREC_FP64, download=False)
        c.orthogonalise(None, download=False)
        c.project(shapes, download=False)
        a, mR = c.alpha(S)
        n0 = c.launches
    G = g["gamma"]
    for s in range(S):
        ref = np.linalg.solve(G, g["beta"][s])
        d = a[s] - ref
        assert np.sqrt(abs(d @ G @ d)) <= 1e-8 * np.sqrt(abs(ref @ G @ ref))
    assert n0 > 10


# ------------------------------------------------------- serial dense form

def _dense_raw(size):
    l = np.arange(size, dtype=np.float64)
    l[0] = 1.0
    raw = np.einsum("i,j,k->ijk", l ** -1.2, l ** -0.7, l ** -1.5)
    return (raw + raw.transpose(1, 2, 0) + raw.transpose(2, 0, 1)) / 3.0


def test_dense_form_vs_reference(mg, golden):
    """modify_bispectrum + calculate_modes on the GPU vs the in-place reference (golden)."""
    g = golden("modes_dense")
    lmax, P = int(g["lmax"]), int(g["P"])
    size = g["modified"].shape[0]
    q, tr, cl = mg.workload(lmax, P)
    mod = mg.modify_bispectrum(_dense_raw(size), np.arange(size), cl[:size])
    nz = g["modified"] != 0
    assert np.array_equal(mod != 0, nz)
    assert np.max(np.abs(mod[nz] - g["modified"][nz]) / np.abs(g["modified"][nz])) <= 1e-14
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        beta = c.calculate_modes(g["modified"])
    assert rel_fro(beta, g["beta"]) <= 1e-12


def test_dense_form_vs_oracle_larger(mg, orc):
    """size beyond lmax (indices above lmax contribute nothing) and P = 6."""
    lmax, P, size = 70, 6, 81
    q, tr, cl = mg.workload(lmax, P)
    cl_ext = np.concatenate([cl, np.full(size - cl.size, cl[-1])])
    mod = mg.modify_bispectrum(_dense_raw(size), np.arange(size), cl_ext)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        beta = c.calculate_modes(mod)
    assert rel_fro(beta, orc.calculate_modes(2, lmax, q, tr, mod)) <= 1e-12


# ------------------------------------------------- late x primordial transfer

def _transfer_inputs(lmax, Pp, xsize):
    xvec = np.linspace(1000.0, 12000.0, xsize)
    l = np.arange(lmax + 1.0)
    qt = np.zeros((xsize, Pp, lmax + 1))
    for xi, x in enumerate(xvec):
        for p in range(Pp):
            qt[xi, p] = np.cos((p + 1) * x / 4000.0) * np.sin(0.1 * l * (1 + p) + x / 3000.0) / (1.0 + l)
    return xvec, qt


@pytest.mark.parametrize("name", ["a", "b"])
def test_transfer_gamma_vs_reference(mg, golden, name):
    """calculate_gamma_2d over all (m, n) on the GPU vs the in-place reference,
    with the reference's asy() nodes: 1e-12."""
    g = golden("gamma_transfer")
    lmax, P, Pp, xsize = (int(v) for v in g["dims_" + name])
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = _transfer_inputs(lmax, Pp, xsize)
    nmu = 3 * lmax // 2 + 1
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        gl = golden("gl_asy")
        if f"x{nmu}" in gl.files:
            c.set_gl(gl[f"x{nmu}"], gl[f"w{nmu}"])
        c.set_transfer(xvec, qt, mg.mode_triples(Pp))
        G = c.gamma_transfer(0.7)
    tol = 1e-12 if f"x{nmu}" in golden("gl_asy").files else 1e-11
    assert rel_max(G, g["gamma_" + name]) <= tol


@pytest.mark.parametrize("name", ["a", "b"])
def test_transfer_gamma_3d_vs_reference(mg, golden, name):
    """calculate_gamma_TTT_3D_nested (gamma_mpi.c's rflag_do3D == 0 path) on the GPU
    vs the in-place reference: 1e-12."""
    g = golden("gamma_3d")
    lmax, P, Pp, xsize = (int(v) for v in g["dims_" + name])
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = mg.transfer_workload(lmax, Pp, xsize)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        c.set_transfer(xvec, qt, mg.mode_triples(Pp))
        G = c.gamma_transfer_3d(float(g["dphi_" + name][0]))
    assert rel_max(G, g["gamma_" + name]) <= 1e-12


def test_transfer_gamma_3d_vs_oracle_rectangular(mg, orc):
    """N late modes != N_prim primordial modes, odd sizes, repeat call identical."""
    lmax, P, Pp, xsize = 90, 5, 3, 41
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = mg.transfer_workload(lmax, Pp, xsize)
    prim = mg.mode_triples(Pp)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        c.set_transfer(xvec, qt, prim)
        G = c.gamma_transfer_3d(0.9)
        G2 = c.gamma_transfer_3d(0.9)
    Go = orc.gamma_3d(2, lmax, q, tr, cl, xvec, qt, prim, 0.9)
    assert G.shape == (len(tr), len(prim))
    assert rel_max(G, Go) <= 1e-12
    assert np.array_equal(G, G2)


def test_transfer_gamma_vs_oracle_wider(mg, orc):
    """Tile edges: N and Nprim not multiples of 32, Pp != P."""
    lmax, P, Pp, xsize = 120, 5, 6, 37
    q, tr, cl = mg.workload(lmax, P)
    xvec, qt = _transfer_inputs(lmax, Pp, xsize)
    prim = mg.mode_triples(Pp)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        c.set_transfer(xvec, qt, prim)
        G = c.gamma_transfer(1.3)
        x, w = c.get_gl()
    Go = orc.gamma_transfer(2, lmax, q, tr, cl, x, w, xvec, qt, prim, 1.3)
    assert rel_max(G, Go) <= 1e-12
