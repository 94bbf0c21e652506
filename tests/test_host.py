"""Host-side logic: synthetic inputs of the benchmark configurations, and the
multi-rank timing of bench.py."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


def _replica_rank(rank, ws, port, out):
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import bench
    td.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got = bench.max_over_ranks([1.0 + rank, 5.0 - rank, 0.5 * rank], ws)
        with open(f"{out}.{rank}", "w") as f:
            f.write(" ".join(repr(v) for v in got))
    finally:
        td.destroy_process_group()


def test_replica_timing_is_max_over_ranks_gloo(tmp_path):
    """bench.py runs one replica per GPU and reports the slowest rank; the
    reduction runs here as two gloo ranks on the CPU."""
    import socket
    import torch.multiprocessing as mp
    sys.path.insert(0, ROOT)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = os.fspath(tmp_path / "r")
    mp.start_processes(_replica_rank, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    for r in range(2):
        vals = [float(v) for v in open(f"{out}.{r}").read().split()]
        assert vals == [2.0, 5.0, 0.5]


def _gamma_shard_rank(rank, ws, port, out):
    import torch
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    for d in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "modal-cmb_gb300")):
        sys.path.insert(0, d)
    import modal_gb300 as mg
    import oracle
    td.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        lmax, P = 60, 6
        q, tr, cl = mg.workload(lmax, P)
        orc = oracle.Oracle()
        nmu = 3 * lmax // 2 + 1
        x, w = orc.gl_nodes(nmu)
        M = orc.mij(orc.legendre_table(x, lmax), 2, lmax, q)
        b, e = mg.mu_shard(nmu, rank, ws)
        part = torch.from_numpy(orc.gamma(np.ascontiguousarray(M[:, :, b:e]), w[b:e], tr))
        td.all_reduce(part, op=td.ReduceOp.SUM)
        np.save(f"{out}.{rank}.npy", part.numpy())
    finally:
        td.destroy_process_group()


def test_gamma_mu_shards_sum_over_ranks_gloo(tmp_path):
    """Gamma shards over the quadrature nodes: two gloo ranks each sum their
    mu_shard of the nodes and one sum all-reduce gives the whole Gamma (the
    oracle computes the partials, so this runs on the CPU)."""
    import socket
    import torch.multiprocessing as mp
    sys.path.insert(0, ROOT)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = os.fspath(tmp_path / "g")
    mp.start_processes(_gamma_shard_rank, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    import modal_gb300 as mg
    import oracle
    lmax, P = 60, 6
    q, tr, cl = mg.workload(lmax, P)
    orc = oracle.Oracle()
    x, w = orc.gl_nodes(3 * lmax // 2 + 1)
    full = orc.gamma(orc.mij(orc.legendre_table(x, lmax), 2, lmax, q), w, tr)
    for r in range(2):
        got = np.load(f"{out}.{r}.npy")
        assert np.max(np.abs(got - full)) <= 1e-13 * np.max(np.abs(full))


def test_max_over_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3, 1.5], 1) == [3.0, 1.5]
