"""Host-side logic: synthetic inputs of the benchmark configurations."""
import numpy as np
import pytest


@pytest.mark.parametrize("P", [1, 2, 5, 10, 30, 40])
def test_mode_triples(mg, P):
    t = mg.mode_triples(P)
    assert len(t) == P * (P + 1) * (P + 2) // 6
    assert len({tuple(r) for r in t.tolist()}) == len(t)
    assert np.all(t[:, 0] <= t[:, 1]) and np.all(t[:, 1] <= t[:, 2]) and t.max() < P
    tot = t.sum(1)
    assert np.all(np.diff(tot) >= 0)  # increasing total order (set_terms_late case 2)


def test_synthetic_inputs(mg, orc):
    q, tr, cl = mg.workload(500, 10)
    assert q.shape == (499, 10) and tr.shape == (220, 3) and np.all(cl > 0)
    raw = mg.legendre_q(2, 500, 10)
    ref = orc.basis_legendre(np.arange(2, 501.0), 9, 2.0, 500.0)
    assert np.max(np.abs(raw - ref)) < 1e-14
    s1 = mg.separable_shapes(500, 3, seed=0)
    s2 = mg.separable_shapes(500, 3, seed=0)
    assert all(np.array_equal(a["tab"], b["tab"]) for a, b in zip(s1, s2))
    b = mg.bump_shapes(5, seed=1)
    assert all(abs(sum(x["c"]) - 1) < 1e-12 and 0.05 <= x["sigma"] <= 0.3 for x in b)
