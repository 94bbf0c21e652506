"""The allocation-free FP64 Gamma entry point (modal_gamma_fp64_noalloc).

It serves callers that must not allocate device memory (engines or graph
executors that own the whole device arena, plugins handed pre-allocated
buffers).  The test allocates the caller's input/output buffers itself (as
such a caller's host would), calls the entry point through the C ABI twice in
a row on different problems, and checks each result against the regular
modal_gamma entry point with the same quadrature.  This file is collected last
so a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest
from conftest import rel_max

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def _call(mg, torch, q, tr, lmin, lmax, nodes=None):
    L = mg.lib()
    dq = _dev(torch, q, np.float64)
    dt = _dev(torch, tr, np.int32)
    N = tr.shape[0]
    dg = torch.full((N, N), float("nan"), dtype=torch.float64, device="cuda")
    if nodes is None:
        dn = dw = None
        nmu = 0
    else:
        dn, dw = _dev(torch, nodes[0], np.float64), _dev(torch, nodes[1], np.float64)
        nmu = nodes[0].size
    vp = ctypes.c_void_p
    st = L.modal_gamma_fp64_noalloc(lmin, lmax, q.shape[1], vp(dq.data_ptr()), N, vp(dt.data_ptr()), nmu,
                                    vp(dn.data_ptr()) if dn is not None else None,
                                    vp(dw.data_ptr()) if dw is not None else None, vp(dg.data_ptr()),
                                    vp(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, dg.cpu().numpy()


def _regular(mg, q, tr, lmin, lmax, nodes=None):
    with mg.Context(0) as c:
        c.set_basis(lmin, lmax, q)
        c.set_modes(tr)
        if nodes is not None:
            c.set_gl(*nodes)
        return c.gamma(mg.PREC_FP64)


def test_noalloc_gamma_matches_regular_entry_point_twice(mg):
    torch = pytest.importorskip("torch")
    cases = [(2, 500, 10, None), (3, 300, 6, "own")]
    for lmin, lmax, P, nodes in cases:
        cl = mg.synthetic_cl(lmax)
        q = mg.weighted_q(mg.legendre_q(lmin, lmax, P), cl, lmin)
        tr = mg.mode_triples(P)
        gl = None
        if nodes == "own":
            gl = mg.gl_nodes(3 * lmax // 2 + 1)
        st, G = _call(mg, torch, q, tr, lmin, lmax, gl)
        assert st == 0, mg.lib().modal_last_error()
        G_ref = _regular(mg, q, tr, lmin, lmax, gl)
        assert np.all(np.isfinite(G))
        assert rel_max(G, G_ref) <= 1e-12


def test_noalloc_rejects_oversize_and_bad_triples(mg):
    torch = pytest.importorskip("torch")
    lmax, P = 2000, 30  # needs ~63 MB of scratch
    q = np.zeros((lmax - 1, P))
    tr = mg.mode_triples(P)
    st, _ = _call(mg, torch, q, tr, 2, lmax)
    assert st == 1
    assert b"scratch" in mg.lib().modal_last_error()
    q, tr, _ = mg.workload(60, 4)
    bad = tr.copy()
    bad[5, 2] = 9
    st, _ = _call(mg, torch, q, bad, 2, 60)
    assert st == 1
    st, G = _call(mg, torch, q, tr, 2, 60)  # the shared scratch still works afterwards
    assert st == 0 and rel_max(G, _regular(mg, q, tr, 2, 60)) <= 1e-12
