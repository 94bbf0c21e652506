"""Split-precision forms against FP64 on the GPU: the tensor-core Gamma (FP16
hi/lo pieces), its node-range partials, and the compensated FP32 projection.
Tolerance: relative Frobenius and relative max error <= 1e-6 (the target for
the split form); emulation predicts ~5e-8."""
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
            assert rel_max(Gs, G64) <= 1e-6, lmax
        nmu = 3 * 200 // 2 + 1
        Sp = c.gamma_partial(mg.PREC_SPLIT, 0, 64) + c.gamma_partial(mg.PREC_SPLIT, 64, nmu)
        assert rel_max(Sp, G64) <= 1e-6


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
    assert rel_fro(Ssp, G64) <= 1e-6 and rel_max(Ssp, G64) <= 1e-6


@pytest.mark.parametrize("lmin,lmax,P", [(2, 40, 1), (2, 60, 4), (2, 500, 10), (3, 600, 17), (2, 700, 20)])
def test_split_gamma_vs_fp64(mg, lmin, lmax, P):
    G64, Gs, Gs2 = _both(mg, lmin, lmax, P)
    assert np.all(np.isfinite(Gs))
    assert rel_fro(Gs, G64) <= 1e-6
    assert rel_max(Gs, G64) <= 1e-6
    assert np.array_equal(Gs, Gs.T)
    assert np.array_equal(Gs, Gs2)  # deterministic


def test_split_gamma_unsorted_duplicate_modes(mg):
    G64, Gs, _ = _both(mg, 2, 300, 6, triples=[[5, 1, 0], [0, 0, 0], [2, 2, 2], [5, 1, 0], [1, 3, 5]])
    assert rel_max(Gs, G64) <= 1e-6


def test_split_gamma_cfg2(mg):
    """Full benchmark size: l <= 2000, P = 30, N = 4960, n_mu = 3001."""
    G64, Gs, _ = _both(mg, 2, 2000, 30)
    assert rel_fro(Gs, G64) <= 1e-6
    assert rel_max(Gs, G64) <= 1e-6


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
    split Gamma within 1e-6 of FP64 (relative Frobenius and max), symmetric and
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
    assert rel_fro(Gs, G64) <= 1e-6 and rel_max(Gs, G64) <= 1e-6
    assert np.array_equal(Gs, Gs.T) and np.array_equal(Gs, Gs2)
    for s in range(2):
        assert rel_fro(bs[s], b64[s]) <= 2e-6, (s, rel_fro(bs[s], b64[s]))
