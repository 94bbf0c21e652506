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


def test_max_over_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3, 1.5], 1) == [3.0, 1.5]
