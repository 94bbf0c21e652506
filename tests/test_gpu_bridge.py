"""The reference-side C bridge (modal-cmb_gb300/bridge/modal_ref_bridge.c)
compiled and linked into a driver that calls the reference's Gamma entry
points (init_orthol_glint, calculate_orthoMij_T, sync_orthoMij,
calculate_orthol) the way ortho_late_mpi.c does; results against the
reference's own calculate_orthol (golden)."""
import os
import subprocess
import sys

import numpy as np
import pytest
from conftest import rel_max

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_golden import pol_inputs  # noqa: E402

pytestmark = pytest.mark.gpu


def _build(tmp_path):
    exe = os.fspath(tmp_path / "bridge_driver")
    lib = os.path.join(ROOT, "modal-cmb_gb300")
    subprocess.run(["gcc", "-O2", "-o", exe, os.path.join(ROOT, "tests", "bridge", "bridge_driver.c"),
                    os.path.join(lib, "bridge", "modal_ref_bridge.c"), "-I" + os.path.join(ROOT, "include"),
                    "-L" + lib, "-lmodal_gb300", "-Wl,-rpath," + lib], check=True)
    return exe


def _run(exe, tmp_path, hdr, arrays, npol, N):
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(np.asarray(hdr, dtype=np.int32).tobytes())
        for a in arrays:
            f.write(np.ascontiguousarray(a).tobytes())
    subprocess.run([exe, os.fspath(inp), os.fspath(out)], check=True)
    return np.fromfile(out, dtype=np.float64).reshape(npol, N, N)


def test_bridge_gamma_matches_reference(mg, golden, tmp_path):
    g = golden("gamma_small")
    lmax, P = int(g["lmax"]), int(g["P"])
    q, tr, cl = mg.workload(lmax, P)
    n = 3 * lmax // 2 + 1
    nodes, weights = golden("gl_asy")[f"x{n}"], golden("gl_asy")[f"w{n}"]
    exe = _build(tmp_path)
    N = len(tr)
    G = _run(exe, tmp_path, [2, lmax, P, N, 0],
             [q.astype(np.float64), tr.astype(np.int32), np.array([n], dtype=np.int32), nodes, weights], 1, N)
    assert rel_max(G[0], g["gamma"]) <= 1e-12
    with mg.Context(0) as c:  # the bridge is the ABI underneath
        c.set_basis(2, lmax, q)
        c.set_modes(tr)
        c.set_gl(nodes, weights)
        c.init_glint()
        assert np.array_equal(G[0], c.gamma())


def test_bridge_polarised_matches_reference(golden, tmp_path):
    g = golden("gamma_pol")
    lmaxT, lmaxE, lminE = (int(v) for v in g["dims"])
    cl, qT, qE, ttt, tte, tee, eee = pol_inputs(lmaxT, lmaxE, lminE)
    exe = _build(tmp_path)
    N = len(ttt)
    hdr = [2, lmaxT, qT.shape[1], N, 1]
    arrays = [qT, ttt.astype(np.int32), np.array([lminE, lmaxE, qE.shape[1]], dtype=np.int32), qE,
              tte.astype(np.int32), tee.astype(np.int32), eee.astype(np.int32),
              np.array([g["nodes"].size], dtype=np.int32), g["nodes"], g["weights"]]
    G = _run(exe, tmp_path, hdr, arrays, 4, N)
    for c in range(4):
        assert rel_max(G[c], g["gamma"][c]) <= 1e-12
