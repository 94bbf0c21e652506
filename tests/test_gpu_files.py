"""The INI-driven GPU drivers (modal_files.ortho_late, gamma_late, modes_late):
Gamma and the orthogonalisation of the modes an INI file describes, the late x
primordial Gamma from the transfer files and the modes of shapes from the
orthol/lambdal files, written as raw FP64 files under the reference's names."""
import os
import sys

import numpy as np
import pytest

import modal_files as mf
from conftest import rel_max

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

pytestmark = pytest.mark.gpu


def test_ortho_late_driver_writes_reference_files(mg, tmp_path):
    lmax, N = 150, 35
    tri = mf._order_case2(N)  # set_terms_late case 2; the basis must cover its largest index
    P = int(tri.max()) + 1
    q, _, cl = mg.workload(lmax, P)
    ini = tmp_path / "run.ini"
    ini.write_text(f"[model]\ndirectory = {tmp_path}/\nT_lmin = 2\nT_lmax = {lmax}\n"
                   f"[basis]\nterms = {N}\norder_late = 2\n[old]\ngflag_pca = 1\n")
    bt = tmp_path / "basis_T.unf"
    mf.array_write(os.fspath(bt), q)
    mf.main(["ortho_late", os.fspath(ini), os.fspath(bt), "--pt", str(P)])
    names = mf.output_names(mf.read_ini(os.fspath(ini)))
    o = mf.array_read(names["orthol_TTT"], N * N).reshape(N, N)
    lam = mf.array_read(names["lambdal_TTT"], N * N).reshape(N, N)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tri)
        c.init_glint()
        g = c.gamma()
        o2, lam2, _, _ = c.orthogonalise(g)
    assert np.array_equal(o, o2) and np.array_equal(lam, lam2)
    assert os.path.basename(names["orthol_TTT"]) == f"orthol_TTT_2-{lmax}_2_{N}"


def _late_ini(tmp_path, lmax, N, extra="", basis_extra="", name="run.ini"):
    ini = tmp_path / name
    ini.write_text(f"[model]\ndirectory = {tmp_path}/\nT_lmin = 2\nT_lmax = {lmax}\ndelta_phi = 0.7\n{extra}"
                   f"[basis]\nterms = {N}\norder_late = 2\norder_prim = 2\n{basis_extra}[old]\ngflag_pca = 1\n")
    return os.fspath(ini)


@pytest.mark.parametrize("do3d", [1, 0])
def test_gamma_late_driver_after_ortho_late(mg, orc, tmp_path, do3d):
    """ortho_late then gamma_late on one INI file: the transfer functions come
    from proj_T files, the lambdal_TTT file from the first run; gamma_TTT holds
    lambdal^T lambdal Gamma with Gamma from the 2D (do3D 1) or 3D (do3D 0) path,
    which matches the oracle to 1e-12."""
    lmax, N, xsize = 70, 12, 23
    # with do3D 0 polarisation is switched on: gamma_late skips it with a warning
    ini = _late_ini(tmp_path, lmax, N, "do_polarisation = 1\n" if do3d == 0 else "", f"do3D = {do3d}\n")
    ini_d = mf.read_ini(ini)
    tri = mf.mode_order(ini_d, N)
    prim, pmax = mf.prim_order(ini_d, N)
    P = int(tri.max()) + 1
    q, _, cl = mg.workload(lmax, P)
    xvec, qt = mg.transfer_workload(lmax, pmax + 1, xsize)
    # read_qtilde reads the E files whenever do_polarisation is 1, as the reference
    mf.write_qtilde(ini_d, xvec, qt, 0.5 * qt if do3d == 0 else None)
    bt, clf = tmp_path / "basis_T.unf", tmp_path / "cl.unf"
    mf.array_write(os.fspath(bt), q)
    mf.array_write(os.fspath(clf), cl)
    if do3d == 0:  # lambdal_TTT from an INI without polarisation (same file names)
        mf.ortho_late(_late_ini(tmp_path, lmax, N, name="ortho.ini"), q)
        with pytest.warns(UserWarning, match="polarisation"):
            out = mf.gamma_late(ini, q, cl)
        for x in ("TTE", "TEE", "EEE"):  # written as zeros, as the reference's 3D path leaves them
            assert np.all(mf.array_read(out.pop(f"gamma_{x}"), N * N) == 0)
    else:
        mf.main(["ortho_late", ini, os.fspath(bt), "--pt", str(P)])
        mf.main(["gamma_late", ini, os.fspath(bt), "--pt", str(P), "--cl", os.fspath(clf)])
        out = {"gamma_TTT": mf.output_names(ini_d)["gamma_TTT"]}
    assert list(out) == ["gamma_TTT"]
    names = mf.output_names(ini_d)
    got = mf.array_read(names["gamma_TTT"], N * N).reshape(N, N)
    lam = mf.array_read(names["lambdal_TTT"], N * N).reshape(N, N)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tri)
        c.set_spectrum(cl)
        c.set_transfer(xvec, qt, prim)
        if do3d == 0:
            G = c.gamma_transfer_3d(0.7)
            Go = orc.gamma_3d(2, lmax, q, tri, cl, xvec, qt, prim, 0.7)
        else:
            G = c.gamma_transfer(0.7)
            x, w = c.get_gl()
            Go = orc.gamma_transfer(2, lmax, q, tri, cl, x, w, xvec, qt, prim, 0.7)
    assert np.array_equal(got, (lam.T @ lam) @ G)
    assert np.max(np.abs(G - Go)) <= 1e-12 * np.max(np.abs(Go))
    assert os.path.basename(names["gamma_TTT"]) == f"gamma_TTT_2-{lmax}_2_2_{N}"


def test_gamma_late_polarised_against_reference(mg, golden, tmp_path):
    """2D path with do_polarisation 1: TTT, TTE, TEE and EEE Gamma files from
    the polarised transfer case (orders from files), each lambdal^T lambdal
    times a Gamma that matches the in-place reference's calculate_gamma_2d."""
    from make_golden import pol_transfer_inputs  # noqa: E402
    d = pol_transfer_inputs()
    g = golden("gamma_transfer_pol")
    lmax, N = d["lmax"], len(d["ttt"])
    for name, t in (("late.txt", d["ttt"]), ("prim.txt", d["prim"]), ("tte.txt", d["tte"]), ("tee.txt", d["tee"]),
                    ("eee.txt", d["eee"])):
        np.savetxt(tmp_path / name, t, fmt="%d")
    ini = tmp_path / "pol.ini"
    ini.write_text(f"[model]\ndirectory = {tmp_path}/\nT_lmin = 2\nT_lmax = {lmax}\nE_lmin = {d['lminE']}\n"
                   f"E_lmax = {d['lmaxE']}\ndo_polarisation = 1\ndelta_phi = {d['dphi']}\nfskyT = {d['fsky_t']}\n"
                   f"fskyE = {d['fsky_e']}\norder_TTT_file_late = late.txt\norder_file_prim = prim.txt\n"
                   f"[basis]\nterms = {N}\norder_late = 3\norder_prim = 3\ndo3D = 1\n[old]\ngflag_pca = 1\n")
    ini = os.fspath(ini)
    ini_d = mf.read_ini(ini)
    orders = [d["tte"], d["tee"], d["eee"]]
    mf.write_qtilde(ini_d, d["xvec"], d["qtT"], d["qtE"])
    mf.ortho_late(ini, d["qT"], d["qE"], orders)
    out = mf.gamma_late(ini, d["qT"], d["cl_total"], d["qE"], orders, d["spec9"])
    assert sorted(out) == ["gamma_EEE", "gamma_TEE", "gamma_TTE", "gamma_TTT"]
    names = mf.output_names(ini_d)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, d["qT"])
        c.set_modes(d["ttt"])
        c.set_spectrum(d["cl_total"])
        c.set_basis_e(d["lminE"], d["lmaxE"], d["qE"])
        c.set_modes_pol(*orders)
        c.set_transfer(d["xvec"], d["qtT"], d["prim"])
        c.set_transfer_pol(d["qtE"], d["spec9"], d["fsky_t"], d["fsky_e"])
        G = [c.gamma_transfer(d["dphi"]), *c.gamma_transfer_pol(d["dphi"])]
    for f, x in enumerate(("TTT", "TTE", "TEE", "EEE")):
        got = mf.array_read(names[f"gamma_{x}"], N * N).reshape(N, N)
        lam = mf.array_read(names[f"lambdal_{x}"], N * N).reshape(N, N)
        assert np.array_equal(got, (lam.T @ lam) @ G[f]), x
        # own GL nodes here, the reference's asy() ones in the golden file
        assert np.max(np.abs(G[f] - g["gamma"][f])) <= 1e-11 * np.max(np.abs(g["gamma"][f])), x


def test_modes_late_driver_from_files(mg, orc, tmp_path):
    """ortho_late (PCA branch, gflag_pca 0) then modes_late from the orthol and
    lambdal files: modes_TTT_<model> holds alpha of each shape, alpha and modesR
    match the oracle's eigenmodetoday restatement (lower triangle of orthol) on
    the file matrices and beta, and a context that orthogonalised itself."""
    lmax, N = 90, 20
    ini = tmp_path / "run.ini"
    ini.write_text(f"[model]\ndirectory = {tmp_path}/\nT_lmin = 2\nT_lmax = {lmax}\nshape1_end = 2\n"
                   f"[basis]\nterms = {N}\norder_late = 2\n[old]\ngflag_pca = 0\n")
    ini = os.fspath(ini)
    tri = mf.mode_order(mf.read_ini(ini), N)
    P = int(tri.max()) + 1
    q, _, cl = mg.workload(lmax, P)
    mf.ortho_late(ini, q)
    shapes = mg.separable_shapes(lmax, 2, seed=3) + mg.bump_shapes(1, seed=4)
    out, a, mR = mf.modes_late(ini, q, cl, shapes, [6, 7, 8])
    names = mf.output_names(mf.read_ini(ini))
    assert sorted(out.values()) == [names["modes_TTT"] + f"_{m}_0" for m in (6, 7, 8)]
    o = mf.array_read(names["orthol_TTT"], N * N).reshape(N, N)
    lam = mf.array_read(names["lambdal_TTT"], N * N).reshape(N, N)
    assert np.count_nonzero(np.triu(o, 1)) > 0  # PCA branch: dense orthol
    with mg.Context(0) as c:
        c.set_basis(2, lmax, q)
        c.set_modes(tri)
        c.set_spectrum(cl)
        c.init_glint()
        c.gamma()
        c.orthogonalise(None, pca_flag=0, download=False)
        beta = c.project(shapes)
        a2, mR2 = c.alpha(len(shapes))
    assert rel_max(a, a2) <= 1e-12 and rel_max(mR, mR2) <= 1e-12
    for s, m in enumerate((6, 7, 8)):
        assert np.array_equal(mf.array_read(out[f"modes_TTT_{m}"], N), a[s])
        a_o, m_o = orc.alpha(o, lam, beta[s])
        assert rel_max(a[s], a_o) <= 1e-10 and rel_max(mR[s], m_o) <= 1e-10


@pytest.mark.parametrize("order_late", [9, 6])
def test_drivers_from_ini_only(mg, tmp_path, order_late):
    """No basis or spectrum file on the command line: the three drivers build
    create_basis_late's table (order_late 9: shifted Legendre plus two
    closed-form columns; 6: Fourier plus eight, scaled by the spectra), take
    the mode lists from the INI's order files (extra-function triples put in)
    and the spectra from its cls / BN / pixel-window tables (load_spectra)."""
    from files_inputs import write_spectrum_tables
    lmax, N, xsize = 80, 15, 21
    raw = mf._order_case2(40)
    np.savetxt(tmp_path / "ttt.txt", raw, fmt="%d")
    keys = write_spectrum_tables(str(tmp_path), lmax, step=1, lmin_tab=0)
    ini = tmp_path / "run.ini"
    ini.write_text(f"[model]\ndirectory = {tmp_path}/\nT_lmin = 2\nT_lmax = {lmax}\ndelta_phi = 0.9\n"
                   f"order_TTT_file_late = ttt.txt\n{keys}[basis]\nterms = {N}\norder_late = {order_late}\n"
                   f"order_prim = 2\n[old]\ngflag_pca = 1\n")
    ini = os.fspath(ini)
    ini_d = mf.read_ini(ini)
    lo = mf.late_orders(ini_d, N)
    pm = lo["pmax_T"] - (2 if order_late == 9 else 8)
    assert lo["ttt"][1].tolist() == [pm + 1, pm + 1, pm + 2]
    sp = mf.load_spectra(ini_d, lens=True)
    B, _ = mf.basis_late(ini_d, lo["pmax_T"], spectra=sp)
    cl = sp["cl_total"]
    prim, pmax = mf.prim_order(ini_d, N)
    xvec, qt = mg.transfer_workload(lmax, pmax + 1, xsize)
    mf.write_qtilde(ini_d, xvec, qt)
    np.save(tmp_path / "tab.npy", mg.separable_shapes(lmax, 1, seed=9)[0]["tab"])
    mf.main(["ortho_late", ini])
    mf.main(["gamma_late", ini])
    mf.main(["modes_late", ini, "--tab", os.fspath(tmp_path / "tab.npy"), "--model", "3"])
    names = mf.output_names(ini_d)
    o = mf.array_read(names["orthol_TTT"], N * N).reshape(N, N)
    gam = mf.array_read(names["gamma_TTT"], N * N).reshape(N, N)
    modes = mf.array_read(names["modes_TTT"] + "_3", N)
    with mg.Context(0) as c:
        c.set_basis(2, lmax, B)
        c.set_modes(lo["ttt"])
        c.set_spectrum(cl)
        c.init_glint()
        o2, lam, _, _ = c.orthogonalise(c.gamma())
        c.set_transfer(xvec, qt, prim)
        G = c.gamma_transfer(0.9)
        beta = c.project([{"kind": mg.SHAPE_SEPARABLE, "tab": np.load(tmp_path / "tab.npy")}])
        a, _ = c.alpha(1, beta)
    assert np.array_equal(o, o2)
    assert np.array_equal(gam, (lam.T @ lam) @ G)
    assert np.array_equal(modes, a[0])


def test_prune_late_driver_matches_prune(mg, golden, tmp_path):
    """prune_late: Gamma and the left-out list from the files the reference's
    pruning driver reads, the elimination order equal to the reference's own
    driver (golden), printed as its lines."""
    import io
    g = golden("basis_prune")
    G, fail, want = g["gamma_a"], g["fail_a"], g["order_a"]
    N = G.shape[0]
    ini = tmp_path / "p.ini"
    ini.write_text(f"[model]\ndirectory = {tmp_path}/\nT_lmax = 100\nE_lmax = 90\n[basis]\nterms = {N}\n"
                   f"order_late = 2\n")
    mf.array_write(os.fspath(tmp_path / f"master_orthol_TTT_100_90_2_{N}.unf"), G)
    (tmp_path / f"faillist_TTT_100_2_{N}.txt").write_text("".join(f"{int(v)}\n" for v in fail))
    buf = io.StringIO()
    order, lam = mf.prune_late(os.fspath(ini), out=buf)
    assert np.array_equal(order, want)
    lines = buf.getvalue().splitlines()
    tri = mf.mode_order(mf.read_ini(os.fspath(ini)), N)
    assert lines[1] == f"modes complete\t{len(fail)}"
    steps = [ln.split("\t") for ln in lines[lines.index("starting reduction") + 1:]]
    assert [int(s[0]) for s in steps] == want.tolist()
    assert all([int(v) for v in s[1:4]] == tri[int(s[0])].tolist() for s in steps)
    assert float(steps[-1][4]) == 1.0
