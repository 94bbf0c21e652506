"""Primordial k-space side on the GPU: grid tetrapyd, Gram matrix
(calculate_ortho) and shape projection (calculate_eigen, integrate_template2)
against the reference in place (golden) and the oracle."""
import os
import sys

import numpy as np
import pytest
from conftest import rel_max

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import prim_inputs  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kmin,kmax_i", [(1, 12), (0, 9), (3, 20), (2, 3), (1, 150)])
def test_prim_points_vs_walk(mg, orc, kmin, kmax_i):
    assert np.array_equal(mg.prim_points(kmin, kmax_i), orc.prim_walk(kmin, kmax_i))


@pytest.mark.parametrize("name", ["a", "b"])
def test_prim_ortho_and_eigen_vs_reference(mg, golden, name):
    g = golden("prim")
    kmin, kmax_i, kmax = g["grid_" + name]
    kmin, kmax_i = int(kmin), int(kmax_i)
    basis, prim, shapes = prim_inputs(kmax_i)
    with mg.Context(0) as c:
        o = c.prim_ortho(kmin, kmax_i, kmax, basis, prim)
        a, n2 = c.prim_eigen(kmin, kmax_i, kmax, basis, prim, shapes)
    assert rel_max(o, g["ortho_" + name]) <= 1e-12
    for n in range(len(shapes)):
        assert rel_max(a[n], g[f"alpha_{name}{n}"]) <= 1e-12
        assert abs(n2[n] - g[f"norm2_{name}{n}"][0]) <= 1e-12 * abs(n2[n])


def test_prim_larger_grid_vs_oracle(mg, orc):
    kmin, kmax_i, kmax, Pp = 1, 160, 0.8, 6
    x = np.arange(kmax_i + 1) / kmax_i
    basis = np.stack([np.cos(np.pi * p * x) + 0.05 * p for p in range(Pp)], axis=1)
    prim = mg.mode_triples(Pp)
    shapes = mg.separable_shapes(kmax_i, 2, 9, 1, 2) + mg.bump_shapes(2, 10)
    for sh in shapes:
        if sh["kind"] == 0:
            sh["tab"][:, :, 0] = 0.0
    with mg.Context(0) as c:
        o = c.prim_ortho(kmin, kmax_i, kmax, basis, prim)
        a, n2 = c.prim_eigen(kmin, kmax_i, kmax, basis, prim, shapes)
    # ~7e5 points: the oracle (like the reference) sums them one by one, whose
    # rounding grows with the count; the GPU sums in blocks.  1e-11 of the largest entry.
    tol = 1e-11
    assert rel_max(o, orc.prim_ortho(kmin, kmax_i, kmax, basis, prim)) <= tol
    for n, sh in enumerate(shapes):
        ar, n2r = orc.prim_eigen(kmin, kmax_i, kmax, basis, prim, sh)
        assert rel_max(a[n], ar) <= tol and abs(n2[n] - n2r) <= tol * abs(n2r)
