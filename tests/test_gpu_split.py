"""Split-precision forms against FP64 on the GPU: the tensor-core Gamma (both
contractions on tcgen05 with exact 7-bit integer slices), its node-range
partials, and the compensated FP32 projection.  Tolerances: the split Gamma
within 1e-12 of the FP64 Gamma (relative Frobenius and max; measured 1.6e-13 at
l <= 2000, P = 30); the FP32 projection within 1e-6; alpha and the kept-subspace
operator lambda^T lambda at PCA floors 1e-6 and 1e-4 within 1e-6."""
import numpy as np
import pytest
from conftest import rel_fro, rel_max

pytestmark = pytest.mark.gpu


def _both(mg, lmin, lmax, P, triples=None):
    cl = mg.synthetic_cl(lmax)
    q = mg.weighted_q(mg.legendre_q(lmin, lmax, P), cl, lmin)
    tr = mg.mode_triples(P) if triples is None else np.asarray(triples, dtype=np.int32)
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(tr)
        G64 = c.gamma(mg.PREC_FP64)
        Gs = c.gamma(mg.PREC_SPLIT)
        Gs2 = c.gamma(mg.PREC_SPLIT)
    return G64, Gs, Gs2


def test_split_projection_many_term_shapes(mg):
    """Separable shapes of more than 4 terms take the FP32 kernel's general
    evaluation (all nine table values per term), next to few-term and bump
    shapes in the same group: <= 1e-6 against FP64, and the captured batch
    gives the same bits as the direct call."""
    lmin, lmax, P = 2, 300, 10
    cl = mg.synthetic_cl(lmax)
    q = mg.weighted_q(mg.legendre_q(lmin, lmax, P), cl, lmin)
    shapes = (mg.separable_shapes(lmax, 3, seed=21, tmin=9, tmax=12) + mg.separable_shapes(lmax, 3, seed=22, tmin=1, tmax=3)
              + mg.bump_shapes(2, seed=23))
    assert any(s["tab"].shape[0] > 8 for s in shapes)
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(mg.mode_triples(P))
        c.set_spectrum(cl)
        b64 = c.project(shapes, mg.PREC_FP64)
        bs = c.project(shapes, mg.PREC_SPLIT)
        bb = c.project_batch(shapes, mg.PREC_SPLIT)
    assert np.array_equal(bs, bb)
    for s in range(len(shapes)):
        assert rel_fro(bs[s], b64[s]) <= 1e-6, (s, rel_fro(bs[s], b64[s]))


def test_split_gamma_after_basis_and_range_changes(mg):
    """One context: the split form's cached tables follow changes of l_max (the
    node count and the K padding) at the same P, and node-range partials after a
    full Gamma."""
    P = 6
    with mg.Context(0) as c:
        for lmax in (300, 700, 200):
            q, tr, cl = mg.workload(lmax, P)
            c.set_basis(2, lmax, q)
            c.set_modes(tr)
            c.init_glint()
            G64 = c.gamma(mg.PREC_FP64)
            Gs = c.gamma(mg.PREC_SPLIT)
            assert rel_max(Gs, G64) <= 1e-12, lmax
        nmu = 3 * 200 // 2 + 1
        Sp = c.gamma_partial(mg.PREC_SPLIT, 0, 64) + c.gamma_partial(mg.PREC_SPLIT, 64, nmu)
        assert rel_max(Sp, G64) <= 1e-12


def test_gamma_partials_over_mu_shards(mg):
    """Gamma over disjoint node ranges (mu_shard of 3 ranks) adds up to Gamma:
    to rounding in FP64, and within the split tolerance in the split form."""
    lmin, lmax, P = 2, 400, 10
    q, tr, cl = mg.workload(lmax, P, lmin)
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(tr)
        c.init_glint()
        G64 = c.gamma(mg.PREC_FP64)
        nmu = 3 * lmax // 2 + 1
        shards = [mg.mu_shard(nmu, r, 3) for r in range(3)]
        S64 = sum(c.gamma_partial(mg.PREC_FP64, b, e) for b, e in shards)
        Ssp = sum(c.gamma_partial(mg.PREC_SPLIT, b, e) for b, e in shards)
        with pytest.raises(mg.ModalError):
            c.gamma_partial(mg.PREC_FP64, 5, 5)
        with pytest.raises(mg.ModalError):  # the device Gamma is a partial now
            c.orthogonalise(None)
    assert rel_max(S64, G64) <= 1e-13
    assert rel_fro(Ssp, G64) <= 1e-12 and rel_max(Ssp, G64) <= 1e-12


@pytest.mark.parametrize("lmin,lmax,P", [(2, 40, 1), (2, 60, 4), (2, 500, 10), (3, 600, 17), (2, 700, 20)])
def test_split_gamma_vs_fp64(mg, lmin, lmax, P):
    G64, Gs, Gs2 = _both(mg, lmin, lmax, P)
    assert np.all(np.isfinite(Gs))
    assert rel_fro(Gs, G64) <= 1e-12
    assert rel_max(Gs, G64) <= 1e-12
    assert np.array_equal(Gs, Gs.T)
    assert np.array_equal(Gs, Gs2)  # deterministic


def test_split_gamma_unsorted_duplicate_modes(mg):
    G64, Gs, _ = _both(mg, 2, 300, 6, triples=[[5, 1, 0], [0, 0, 0], [2, 2, 2], [5, 1, 0], [1, 3, 5]])
    assert rel_max(Gs, G64) <= 1e-12


def test_split_gamma_cfg2_alpha_basis_with_floor(mg):
    """Full benchmark size, l <= 2000, P = 30 (N = 4960, n_mu = 3001): the split
    Gamma within 1e-12 of FP64; then each Gamma through the same FP64
    orthogonalisation with a PCA floor (1e-6, 1e-4 of e_max): the same kept rank,
    alpha = lambda^T lambda beta within 1e-6, and the kept-subspace operator
    lambda^T lambda (the reference's orthoinv, eigenmodetoday_mpi.c:148-162)
    within 1e-6 on random probes.  The reference's floor-free rule keeps
    eigenvalues down to ~1e-13 e_max and is ill-posed at this size (two FP64
    solvers differ by ~1e-5 there), hence the floors."""
    lmax, P = 2000, 30
    q, tr, cl = mg.workload(lmax, P)
    rng = np.random.default_rng(7)
    probes = rng.standard_normal((4, len(tr)))
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        c.init_glint()
        G64 = c.gamma(mg.PREC_FP64)
        Gs = c.gamma(mg.PREC_SPLIT)
        assert rel_fro(Gs, G64) <= 1e-12 and rel_max(Gs, G64) <= 1e-12
        beta = c.project(mg.separable_shapes(lmax, 4, seed=3), mg.PREC_FP64)
        for floor in (1e-6, 1e-4):
            c.set_pca_floor(floor)
            out = []
            for G in (G64, Gs):
                _, lam, branch, rank = c.orthogonalise(G)
                a, _ = c.alpha(4, beta)
                out.append((rank, a, (lam.T @ (lam @ probes.T)).T))
            (r64, a64, p64), (rs, as_, ps) = out
            assert rs == r64, floor
            assert rel_fro(as_, a64) <= 1e-6, floor
            assert rel_fro(ps, p64) <= 1e-6, floor
        c.set_pca_floor(0.0)


def test_split_projection_bumps_cfg3(mg):
    """cfg3's non-separable shapes at full size (l <= 2000, P = 30): 16 Gaussian
    bumps, sigma from 0.05 to 0.3, in FP32 against FP64, <= 1e-6 each."""
    lmax, P = 2000, 30
    q, tr, cl = mg.workload(lmax, P)
    shapes = mg.bump_shapes(14, seed=33)
    shapes += [{"kind": mg.SHAPE_BUMP, "c": np.array([0.34, 0.33, 0.33]), "sigma": 0.05},
               {"kind": mg.SHAPE_BUMP, "c": np.array([0.5, 0.3, 0.2]), "sigma": 0.05}]
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        b64 = c.project(shapes, mg.PREC_FP64)
        bs = c.project(shapes, mg.PREC_SPLIT)
    for s in range(len(shapes)):
        assert rel_fro(bs[s], b64[s]) <= 1e-6, (s, shapes[s]["sigma"], rel_fro(bs[s], b64[s]))


@pytest.mark.parametrize("lmin,lmax,P,S", [(2, 60, 4, 3), (2, 500, 10, 9), (5, 300, 33, 5), (2, 800, 40, 6)])
def test_split_projection_vs_fp64(mg, lmin, lmax, P, S):
    """FP32 slab kernel (compensated sums) against the FP64 one: <= 1e-6 relative."""
    cl = mg.synthetic_cl(lmax)
    q = mg.weighted_q(mg.legendre_q(lmin, lmax, P), cl, lmin)
    tr = mg.mode_triples(P)
    shapes = mg.separable_shapes(lmax, (S + 1) // 2, seed=5, tmin=1, tmax=4) + mg.bump_shapes(S // 2, seed=6)
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        b64 = c.project(shapes, mg.PREC_FP64)
        bs = c.project(shapes, mg.PREC_SPLIT)
        bs2 = c.project(shapes, mg.PREC_SPLIT)
    assert np.array_equal(bs, bs2)
    # 1e-6 up to P = 32 (the benchmark's P = 30); at P = 40 the FP32 sums over
    # 32-point blocks of degree-39 polynomials cancel more: 2e-6 (measured 1.4e-6
    # for the sharpest bump, sigma ~ 0.05).
    tol = 1e-6 if P <= 32 else 2e-6
    for s in range(S):
        assert rel_fro(bs[s], b64[s]) <= tol, (s, rel_fro(bs[s], b64[s]))


def test_split_cfg5_largest_config(mg):
    """The largest configuration, l <= 2500, P = 40 (N = 11480, n_mu = 3751):
    split Gamma within 1e-12 of FP64 (relative Frobenius and max), symmetric and
    reproducible; two shapes projected in FP32 within the P = 40 bound (2e-6)
    of FP64."""
    lmax, P = 2500, 40
    q, tr, cl = mg.workload(lmax, P)
    shapes = mg.separable_shapes(lmax, 1, seed=51, tmin=2, tmax=2) + mg.bump_shapes(1, seed=52)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_spectrum(cl)
        c.init_glint()
        G64 = c.gamma(mg.PREC_FP64)
        Gs = c.gamma(mg.PREC_SPLIT)
        Gs2 = c.gamma(mg.PREC_SPLIT)
        b64 = c.project(shapes, mg.PREC_FP64)
        bs = c.project(shapes, mg.PREC_SPLIT)
    assert G64.shape == (11480, 11480)
    assert rel_fro(Gs, G64) <= 1e-12 and rel_max(Gs, G64) <= 1e-12
    assert np.array_equal(Gs, Gs.T) and np.array_equal(Gs, Gs2)
    for s in range(2):
        assert rel_fro(bs[s], b64[s]) <= 2e-6, (s, rel_fro(bs[s], b64[s]))


@pytest.mark.parametrize("lmin,lmax,P,S", [(2, 40, 1, 1), (2, 61, 5, 7), (3, 257, 12, 9), (2, 600, 32, 6)])
def test_split_projection_tensor_cores(mg, lmin, lmax, P, S):
    """The tensor-core slab kernel (P <= 32, switched on) against FP64
    (<= 1e-6 relative per shape) and against the CUDA-core FP32 kernel; groups
    of four shapes that mix kinds and term counts (up to 12 terms, past the
    4-term row-coefficient path), an S that is not a multiple of 4, odd and even
    l_min, one-function bases; repeated calls and the captured batch give the
    same bits."""
    cl = mg.synthetic_cl(lmax)
    q = mg.weighted_q(mg.legendre_q(lmin, lmax, P), cl, lmin)
    shapes = (mg.separable_shapes(lmax, (S + 1) // 2, seed=41, tmin=1, tmax=12 if S > 5 else 3)
              + mg.bump_shapes(S // 2, seed=42))
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(mg.mode_triples(P))
        c.set_spectrum(cl)
        assert not c.proj_kernel()  # the CUDA-core kernel by default
        c.set_proj_kernel(True)
        assert c.proj_kernel()
        b64 = c.project(shapes, mg.PREC_FP64)
        bt = c.project(shapes, mg.PREC_SPLIT)
        bt2 = c.project(shapes, mg.PREC_SPLIT)
        bb = c.project_batch(shapes, mg.PREC_SPLIT)
        c.set_proj_kernel(False)
        bc = c.project(shapes, mg.PREC_SPLIT)
    assert np.array_equal(bt, bt2) and np.array_equal(bt, bb)
    for s in range(S):
        assert rel_fro(bt[s], b64[s]) <= 1e-6, (s, rel_fro(bt[s], b64[s]))
        assert rel_fro(bt[s], bc[s]) <= 2e-6, (s, rel_fro(bt[s], bc[s]))


def test_split_projection_kernel_choice(mg):
    """The CUDA-core kernel by default; switched on, P <= 32 projects on the
    tensor cores and P > 32 stays on the CUDA-core kernel."""
    for P, want in ((32, True), (33, False)):
        lmax = 120
        q, tr, cl = mg.workload(lmax, P)
        with mg.Context(0) as c:
            c.set_basis(2, lmax, q)
            c.set_modes(tr)
            c.set_spectrum(cl)
            assert not c.proj_kernel()
            c.set_proj_kernel(True)
            assert c.proj_kernel() == want
            c.set_proj_kernel(False)
            assert not c.proj_kernel()
            assert mg.lib().modal_set_proj_kernel(c.h, 2) != 0  # only 0 or 1
