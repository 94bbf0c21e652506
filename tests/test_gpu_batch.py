"""Graph-captured batched projection and the launch-configuration tuner."""
import os

import numpy as np
from conftest import rel_fro
import pytest

pytestmark = pytest.mark.gpu


def _ctx(mg, lmax=160, P=6):
    q, tr, cl = mg.workload(lmax, P)
    c = mg.Context(0)
    c.set_basis(2, lmax, q)
    c.set_modes(tr)
    c.set_spectrum(cl)
    return c


def _mixed(mg, lmax, seed, S=10):
    return mg.config_shapes(lmax, ("mix", S, 1, 3), seed=seed)


def _same_layout(mg, shapes):
    """New values, same kinds and term counts."""
    out = []
    for sh in shapes:
        if sh["kind"] == mg.SHAPE_SEPARABLE:
            out.append({"kind": sh["kind"], "tab": sh["tab"] * 0.5 + 0.1})
        else:
            c = np.roll(np.asarray(sh["c"]), 1)
            out.append({"kind": sh["kind"], "c": c, "sigma": sh["sigma"] * 1.1})
    return out


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_equals_project_and_replays(mg, prec):
    lmax = 160
    with _ctx(mg, lmax) as c:
        a = _mixed(mg, lmax, 1)
        b = _same_layout(mg, a)
        ref_a = c.project(a, prec)
        ref_b = c.project(b, prec)
        n0 = c.captures
        got_a = c.project_batch(a, prec)
        assert c.captures == n0 + 1
        l0 = c.launches
        got_b = c.project_batch(b, prec)
        assert c.captures == n0 + 1  # replayed, not re-captured
        assert c.launches > l0
        assert np.array_equal(got_a, ref_a) and np.array_equal(got_b, ref_b)
        # the batch's beta stays on the device for alpha
        c.init_glint()
        c.gamma(mg.PREC_FP64, download=False)
        c.orthogonalise(None, download=False)
        c.project_batch(b, prec)
        al1, _ = c.alpha(len(b))
        al2, _ = c.alpha(len(b), ref_b)
        assert np.array_equal(al1, al2)


def test_batch_recaptures_on_layout_or_buffer_change(mg):
    lmax = 160
    with _ctx(mg, lmax) as c:
        a = _mixed(mg, lmax, 3)
        c.project_batch(a, 1)
        n = c.captures
        c.project_batch(a[:-1], 1)  # new S
        assert c.captures == n + 1
        big = mg.config_shapes(lmax, ("mix", 64, 1, 4), seed=5)
        c.project(big, 0)  # grows the shared scratch and shape tables
        got = c.project_batch(a, 1)
        assert c.captures == n + 2
        assert np.array_equal(got, c.project(a, 1))


def test_autotune_applies_and_caches(mg, tmp_path):
    """The tuner picks between the tensor-core kernel and the CUDA-core FP32
    kernel's launch configurations, caches its choice and reads it back.  A
    CUDA-core configuration changes the schedule, not the arithmetic (same bits
    for every one); the two kernels agree within the FP32 tolerance."""
    lmax = 200
    path = os.fspath(tmp_path / "tune.txt")
    with _ctx(mg, lmax, 8) as c:
        shapes = _mixed(mg, lmax, 7, 12)
        assert not c.proj_kernel()  # the CUDA-core kernel by default
        before_cc = c.project(shapes, 1)
        c.set_proj_kernel(True)
        assert c.proj_kernel()
        before_tc = c.project(shapes, 1)
        c.set_proj_kernel(False)
        b64 = c.project(shapes, 0)
        for s in range(len(shapes)):
            assert rel_fro(before_tc[s], b64[s]) <= 1e-6 and rel_fro(before_cc[s], b64[s]) <= 1e-6
        t = c.autotune(path)
        assert t["proj_tc"] in (0, 1) and t["gamma_kc"] in (4, 8, 16, 32)
        if not t["proj_tc"]:
            assert t["proj_sg"] in (4, 8) and t["proj_cpb"] in (0, 1, 2)
        assert np.array_equal(c.project(shapes, 1), before_tc if t["proj_tc"] else before_cc)
        g1 = c.gamma(mg.PREC_FP64)
    lines = open(path).read().splitlines()
    assert len(lines) == 2 and lines[0].startswith("proj2 sm_") and lines[1].startswith("gamma64 sm_")
    with _ctx(mg, lmax, 8) as c2:
        assert c2.autotune(path) == t  # read back, not re-timed
        assert len(open(path).read().splitlines()) == 2
        c2.init_glint()
        assert np.array_equal(c2.gamma(mg.PREC_FP64), g1)
    # every candidate, forced through the cache file, gives its kernel's beta
    key = lines[0].split("  #")[0].rsplit(" ", 3)[0]
    for n, (sg, cpb, tcv) in enumerate([(4, 0, 0), (8, 1, 0), (4, 2, 0), (8, 0, 0), (0, 0, 1)]):
        p2 = os.fspath(tmp_path / f"t{n}.txt")
        with open(p2, "w") as f:
            f.write(f"{key} {sg} {cpb} {tcv}\n{lines[1]}\n")
        with _ctx(mg, lmax, 8) as c3:
            got = c3.autotune(p2)
            assert (got["proj_sg"], got["proj_cpb"], got["proj_tc"]) == (sg, cpb, tcv)
            ref = before_tc if tcv else before_cc
            assert np.array_equal(c3.project(shapes, 1), ref)
            assert np.array_equal(c3.project_batch(shapes, 1), ref)
