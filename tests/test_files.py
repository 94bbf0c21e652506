"""Reference-compatible INI parsing, file names, raw arrays and mode orders
(modal-cmb_gb300/modal_files.py), against the conventions of parameter.c,
arrays.c, io.c and set_terms_late; the GPU driver end to end is in
test_gpu_files.py."""
import os
import sys

import numpy as np
import pytest

import modal_files as mf

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from files_inputs import CASES, qtilde_tables, write_case, write_spectrum_tables  # noqa: E402

write_spectrum_files = write_spectrum_tables  # also used by the GPU driver tests

INI = """
; comment line
[model]
directory = "{d}"   ; trailing comment
T_lmin = 2
T_lmax = 2000
E_lmin = 3
E_lmax = 1500
do_polarisation = 0
[basis]
terms = 4960
order_prim = 3
order_late = 2
orthol_file = orthol
# another comment
gamma_file = gamma
[old]
gflag_pca = 1
"""


def _ini(tmp_path):
    p = tmp_path / "run.ini"
    p.write_text(INI.format(d=str(tmp_path) + "/"))
    return os.fspath(p)


def test_read_ini_keys(tmp_path):
    ini = mf.read_ini(_ini(tmp_path))
    assert ini["model:directory"] == str(tmp_path) + "/"
    assert mf.getint(ini, "model:T_lmax", 0) == 2000
    assert mf.getint(ini, "basis:terms", 0) == 4960
    assert mf.getint(ini, "model:missing", 7) == 7
    assert mf.getstring(ini, "basis:orthol_file", "") == "orthol"


def test_output_names_follow_parameter_c(tmp_path):
    d = str(tmp_path) + "/"
    names = mf.output_names(mf.read_ini(_ini(tmp_path)))
    # parameter.c: directory + name + _XXX_ + T range [+ _ + E range] + _order_late + _terms
    assert names["orthol_TTT"] == d + "orthol_TTT_2-2000_2_4960"
    assert names["orthol_TTE"] == d + "orthol_TTE_2-2000_3-1500_2_4960"
    assert names["orthol_TEE"] == d + "orthol_TEE_2-2000_3-1500_2_4960"
    assert names["orthol_EEE"] == d + "orthol_EEE_3-1500_2_4960"
    assert names["lambdal_TTT"] == d + "lambdal_TTT_2-2000_2_4960"
    assert names["modes_EEE"] == d + "modes_EEE_3-1500_2_4960"
    # gamma carries the primordial order too
    assert names["gamma_TTT"] == d + "gamma_TTT_2-2000_3_2_4960"
    assert names["gamma_TTE"] == d + "gamma_TTE_2-2000_3-1500_3_2_4960"


def test_raw_arrays_and_triples(tmp_path):
    a = np.random.default_rng(1).standard_normal((7, 5))
    p = os.fspath(tmp_path / "a.unf")
    mf.array_write(p, a)
    assert os.path.getsize(p) == 7 * 5 * 8
    assert np.array_equal(mf.array_read(p, 35).reshape(7, 5), a)
    with pytest.raises(ValueError):
        mf.array_read(p, 36)
    t = tmp_path / "order.txt"
    t.write_text("0 0 0\n0 0 1\n0 1 1\n")
    assert mf.load_three_int(os.fspath(t)).tolist() == [[0, 0, 0], [0, 0, 1], [0, 1, 1]]


def test_mode_orders(mg):
    c2 = mf._order_case2(200)
    assert c2[:7].tolist() == [[0, 0, 0], [0, 0, 1], [0, 1, 1], [0, 0, 2], [1, 1, 1], [0, 1, 2], [0, 0, 3]]
    s = c2.sum(1)
    assert np.all(np.diff(s) >= 0) and len({tuple(r) for r in c2.tolist()}) == 200
    assert np.all(c2[:, 0] <= c2[:, 1]) and np.all(c2[:, 1] <= c2[:, 2])
    for P in (4, 6):  # the benchmark's lists are case 2 restricted to indices < P
        want = mg.mode_triples(P)
        got = np.array([r for r in mf._order_case2(400).tolist() if max(r) < P][:len(want)])
        assert np.array_equal(got, want)
    c1 = mf._order_case1(12)
    assert len({tuple(r) for r in c1.tolist()}) == 12


def test_prim_orders(tmp_path):
    d = str(tmp_path) + "/"
    (tmp_path / "prim.txt").write_text("0 0 0\n0 0 1\n0 1 1\n1 1 1\n0 0 2\n")
    base = f"[model]\ndirectory = {d}\norder_file_prim = prim.txt\n[basis]\n"
    for case, want in [(2, mf._order_case2(4).tolist()), (1, mf._order_case1(4).tolist()),
                       (3, [[0, 0, 0], [0, 0, 1], [0, 1, 1], [1, 1, 1]]),
                       # case 4: N-1 file triples, (pmax+1, pmax+1, pmax+2) put in at index 1
                       (4, [[0, 0, 0], [2, 2, 3], [0, 0, 1], [0, 1, 1]])]:
        (tmp_path / "p.ini").write_text(base + f"order_prim = {case}\n")
        t, pm = mf.prim_order(mf.read_ini(os.fspath(tmp_path / "p.ini")), 4)
        assert t.tolist() == want and pm == max(r[2] for r in want), case
    (tmp_path / "p.ini").write_text(base + "order_prim = 3\n")
    with pytest.raises(ValueError):
        mf.prim_order(mf.read_ini(os.fspath(tmp_path / "p.ini")), 6)


def test_proj_names_follow_parameter_c(tmp_path):
    d = str(tmp_path) + "/"
    names = mf.proj_names(mf.read_ini(_ini(tmp_path)))
    # parameter.c:725-760: directory + proj + _T_ + T_lmax + _ + order_prim; sizes without the order
    assert names == {"T_data": d + "proj_T_2000_3", "E_data": d + "proj_E_1500_3",
                     "T_size": d + "proj_T_2000_size", "E_size": d + "proj_E_1500_size"}
    (tmp_path / "abs.ini").write_text("[basis]\nproj_file = /data/tr\n")
    names = mf.proj_names(mf.read_ini(os.fspath(tmp_path / "abs.ini")))
    assert names == {"T_data": "/data/tr_T", "E_data": "/data/tr_E", "T_size": "/data/tr_T_size",
                     "E_size": "/data/tr_E_size"}


@pytest.mark.parametrize("order_prim,pol", [(3, False), (4, True)])
def test_qtilde_files_round_trip(tmp_path, order_prim, pol):
    """write_qtilde lays the files out as output_qtilde (size file of two native
    ints, row 0 = x grid, column 0 = l); read_qtilde gives back the
    [xsize][P][lsize] table, with order_prim 4 through the _l1/_l2 pair."""
    d = str(tmp_path) + "/"
    (tmp_path / "t.ini").write_text(f"[model]\ndirectory = {d}\nT_lmax = 30\nE_lmax = 30\n"
                                    f"do_polarisation = {int(pol)}\n[basis]\norder_prim = {order_prim}\n")
    ini = mf.read_ini(os.fspath(tmp_path / "t.ini"))
    rng = np.random.default_rng(3)
    xs, P, L = 9, 4, 31
    x = np.linspace(10.0, 90.0, xs)
    qT, qE = rng.standard_normal((xs, P, L)), rng.standard_normal((xs, P, L))
    names = mf.write_qtilde(ini, x, qT, qE if pol else None)
    assert np.fromfile(names["T_size"], dtype=np.int32).tolist() == [L + 1, xs + 1]
    sfx = ["0", "1", "l1", "l2"] if order_prim == 4 else ["0", "1", "2", "3"]
    for n, sx in enumerate(sfx):
        raw = mf.array_read(f"{names['T_data']}_{sx}").reshape(L + 1, xs + 1)
        assert raw[0, 0] == n and np.array_equal(raw[0, 1:], x) and np.array_equal(raw[1:, 0], np.arange(L))
        assert np.array_equal(raw[5, 3], qT[2, n, 4])  # data[l+1][i+1] = q~_n(l, x_i)
    got = mf.read_qtilde(ini, P - 1)
    assert np.array_equal(got["x"], x) and np.array_equal(got["lvec_T"], np.arange(L))
    assert np.array_equal(got["qt_T"], qT)
    if pol:
        assert np.array_equal(got["qt_E"], qE)
    else:
        assert "qt_E" not in got
    with pytest.raises(FileNotFoundError):  # a missing index file is an error, not a short table
        os.remove(f"{names['T_data']}_{sfx[-1]}")
        mf.read_qtilde(ini, P - 1)


def test_modes_suffix_follows_output_modes(tmp_path):
    """output_modes names the file _<model> then one _<p> per shape parameter up
    to the last one with a non-zero model:shapeX_end (0 where its own end is 0)."""
    cases = [("", 7, "_7"), ("shape1_end = 3\n", 7, "_7_1"), ("shape2_end = 3\n", 999, "_999_0_2"),
             ("shape1_end = 1\nshape3_end = 5\n", 998, "_998_1_0_3")]
    for body, model, want in cases:
        (tmp_path / "m.ini").write_text("[model]\n" + body)
        ini = mf.read_ini(os.fspath(tmp_path / "m.ini"))
        assert mf.modes_suffix(ini, model, 1, 2, 3) == want, body


def _order_ini(tmp_path, case, N_file, pol=False):
    d = str(tmp_path) + "/"
    raw = mf._order_case2(N_file)
    np.savetxt(tmp_path / "ttt.txt", raw, fmt="%d")
    np.savetxt(tmp_path / "tte.txt", raw[:, [0, 1, 2]] % 3, fmt="%d")
    np.savetxt(tmp_path / "tee.txt", np.stack([raw[:, 1] % 2, raw[:, 2] % 2, raw[:, 0]], 1), fmt="%d")
    np.savetxt(tmp_path / "eee.txt", raw % 4, fmt="%d")
    (tmp_path / "o.ini").write_text(
        f"[model]\ndirectory = {d}\ndo_polarisation = {int(pol)}\norder_TTT_file_late = ttt.txt\n"
        f"order_TTE_file_late = tte.txt\norder_TEE_file_late = tee.txt\norder_EEE_file_late = eee.txt\n"
        f"[basis]\norder_late = {case}\n")
    return mf.read_ini(os.fspath(tmp_path / "o.ini")), raw


def test_late_orders_shift_and_extra_terms(tmp_path):
    """set_terms_late: orders 4-7, 9 and 10 read the file shifted down and put
    their extra-function triples (offsets from pmax_T) in the freed rows."""
    N = 12
    for case, k, rows, add in [(3, 0, {}, 0), (8, 0, {}, 0), (4, 1, {1: (1, 1, 2)}, 2), (7, 1, {1: (1, 1, 2)}, 2),
                               (9, 1, {1: (1, 1, 2)}, 2), (5, 3, {1: (1, 1, 1), 2: (2, 2, 3), 3: (4, 4, 5)}, 5),
                               (6, 4, {1: (1, 1, 2), 2: (3, 5, 8), 3: (3, 6, 7), 4: (4, 5, 6)}, 8),
                               (10, 3, {0: (2, 2, 4), 1: (1, 3, 4), 2: (1, 1, 5)}, 5)]:
        ini, raw = _order_ini(tmp_path, case, N)
        lo = mf.late_orders(ini, N)
        t = lo["ttt"]
        # untouched rows: the file's row n - k above the shift (n >= k for order 10), row n below it
        first = k if case == 10 else k + 1
        for n in range(N):
            if n in rows:
                continue
            want = raw[n - k] if (k and n >= first) else raw[n]
            assert t[n].tolist() == want.tolist(), (case, n)
        shifted = np.array([raw[n - k] if (k and n >= first) else raw[n] for n in range(N)])
        pm = int(shifted[:, 2].max())
        for n, offs in rows.items():
            assert t[n].tolist() == [pm + o for o in offs], (case, n)
        assert lo["pmax_T"] == pm + add, case
    ini, raw = _order_ini(tmp_path, 3, N)
    with pytest.raises(ValueError):
        mf.late_orders(ini, N + 1)
    with pytest.raises(ValueError):
        mf.late_orders(mf.read_ini(os.fspath(tmp_path / "o.ini")) | {"basis:order_late": "11"}, N)


def test_late_orders_polarised_files(tmp_path):
    """TTE and EEE lines are the triples; a TEE line (a, b, c) is (c, a, b), T
    index first (fixed_data.c:343-349); pmax_T/pmax_E count the T and E
    entries."""
    N = 10
    ini, raw = _order_ini(tmp_path, 2, N, pol=True)
    lo = mf.late_orders(ini, N)
    assert lo["ttt"].tolist() == mf._order_case2(N).tolist()
    tee_file = np.loadtxt(tmp_path / "tee.txt", dtype=int)
    assert lo["tee"].tolist() == tee_file[:, [2, 0, 1]].tolist()
    assert lo["tte"].tolist() == (raw % 3).tolist() and lo["eee"].tolist() == (raw % 4).tolist()
    assert lo["pmax_T"] == max(raw[:, 2].max(), (raw[:, 1] % 3).max(), lo["tee"][:, 0].max())
    assert lo["pmax_E"] == max((raw[:, 2] % 3).max(), lo["tee"][:, 2].max(), (raw[:, 2] % 4).max())
    lo2 = mf.late_orders(ini, N, pol_lists=(lo["tte"], lo["tee"], lo["eee"]))
    assert all(np.array_equal(lo[k], lo2[k]) for k in ("tte", "tee", "eee"))


def test_basis_families_match_reference(golden):
    """basis_functions.c compiled in place: Legendre, Fourier and sin-log
    bit for bit (the same libm calls in the same order); the 'bi' family,
    restated from its definition, to 1e-12 up to degree 7, beyond which the
    reference's monomial evaluation loses digits (next test)."""
    g = golden("basis_families")
    for name in "ab":
        lo, hi, pmax, vmin = g["dims_" + name]
        v = np.arange(lo, hi + 1, dtype=np.float64)
        for fam, fn in (("legendre", mf.basis_legendre), ("fourier", mf.basis_fourier),
                        ("sinlog", mf.basis_sinlog)):
            assert np.array_equal(fn(v, int(pmax), float(vmin), float(hi)), g[f"{fam}_{name}"]), (name, fam)
        bi, ref = mf.basis_bi(v, int(pmax), float(vmin), float(hi)), g["bi_" + name]
        for j in range(8):
            assert np.max(np.abs(bi[:, j] - ref[:, j])) <= 1e-12 * np.max(np.abs(ref[:, j])), (name, j)


def test_bi_family_orthonormal():
    """Known answer for the 'bi' polynomials: orthonormal on [0, 1] under the
    weight 2x - 3x^2/2 (a 64-point Gauss rule is exact here) to 1e-13
    through degree 30, with p_0 = sqrt 2 and positive leading coefficients."""
    x, w = np.polynomial.legendre.leggauss(64)
    t = (x + 1.0) / 2.0
    wt = w / 2.0 * (2.0 * t - 1.5 * t * t)
    B = mf.basis_bi(t, 30, 0.0, 1.0)
    G = (B * wt[:, None]).T @ B
    assert np.max(np.abs(G - np.eye(31))) <= 1e-13
    assert np.allclose(B[:, 0], np.sqrt(2.0), rtol=0, atol=1e-15)
    assert np.all(np.diff(B[-3:, 30]) > 0)  # increasing towards x = 1 (positive leading coefficient)


@pytest.mark.parametrize("case", [1, 4, 6, 7, 8, 9, 10])
def test_basis_late_columns(tmp_path, case):
    """create_basis_late's tables: the family columns, and the appended
    closed-form columns of orders 4, 6, 7, 9 and 10 (row 0 zero except for
    order 9), checked entry by entry against the formulas."""
    import math
    lmin, lmax, n = 2, 300, 12
    (tmp_path / "b.ini").write_text(f"[model]\nT_lmin = {lmin}\nT_lmax = {lmax}\ndo_polarisation = 1\n"
                                    f"E_lmin = 3\nE_lmax = 200\n[basis]\norder_late = {case}\n")
    ini = mf.read_ini(os.fspath(tmp_path / "b.ini"))
    l = np.arange(lmax + 1.0)
    spectra = {"cl_tt": 1.0 / (1.0 + l * l), "noise_tt": 1e-6 + 0 * l, "beam_tt": np.exp(-l * 1e-3),
               "cl_tp": 0.1 / (2.0 + l)}
    B, E = mf.basis_late(ini, n, 5, spectra if case == 6 else None)
    T = np.arange(lmin, lmax + 1.0)
    assert B.shape == (T.size, n + 1) and E.shape == (198, 6)
    fam = {1: mf.basis_bi, 4: mf.basis_fourier, 6: mf.basis_fourier, 7: mf.basis_bi, 8: mf.basis_sinlog,
           9: mf.basis_legendre, 10: mf.basis_legendre}[case]
    nfam = {1: n + 1, 4: n - 1, 6: n - 7, 7: n - 1, 8: n + 1, 9: n - 1, 10: n - 4}[case]
    assert np.array_equal(B[:, :nfam], fam(T, nfam - 1, float(lmin), float(lmax)))
    efam = {1: mf.basis_bi, 4: mf.basis_fourier, 6: mf.basis_fourier, 7: mf.basis_bi, 8: mf.basis_sinlog,
            9: mf.basis_legendre, 10: mf.basis_legendre}[case]
    assert np.array_equal(E, efam(np.arange(3, 201.0), 5, 3.0, 200.0))
    i = 57
    x = T[i] * (T[i] + 1) / (lmax * (lmax + 1.0))
    z, wv = math.sqrt(x), math.pow((2 * T[i] + 1) / (2 * lmax + 1.0), 1 / 6)
    if case in (4, 7, 9):
        assert B[i, n - 1] == wv / z and B[i, n] == wv * z
        assert (B[0, n - 1] == 0 and B[0, n] == 0) == (case != 9)
    if case == 6:
        li = int(T[i])
        c = wv / math.sqrt(spectra["cl_tt"][li] + spectra["noise_tt"][li] / spectra["beam_tt"][li] ** 2)
        want = [wv / z, wv * z, c, c * x, c * spectra["cl_tt"][li], c * spectra["cl_tp"][li],
                c * x * spectra["cl_tt"][li], c * x * spectra["cl_tp"][li]]
        assert np.allclose(B[i, n - 7:], want, rtol=1e-15, atol=0) and np.all(B[0, n - 7:] == 0)
    if case == 10:
        l1 = T[i] / lmax
        want = [wv / (l1 * z), wv / z, wv * l1 / z, wv * z, wv * l1 * l1 * z]
        assert np.allclose(B[i, n - 4:], want, rtol=1e-15, atol=0)
    with pytest.raises(ValueError):
        (tmp_path / "c.ini").write_text("[model]\nT_lmax = 50\n[basis]\norder_late = 5\n")
        mf.basis_late(mf.read_ini(os.fspath(tmp_path / "c.ini")), 8)


def test_load_spectra_tables(tmp_path):
    """load_cl / load_BN / load_lens / load_TL: D_l -> 2 pi D_l/(l(l+1)) on the
    tabulated l exactly, natural-spline values in between (scipy's natural
    CubicSpline to 1e-13), the pixel window by row, zeros below the first
    tabulated l, TE beam sqrt(b_T b_E) and noise 0, PT/l^3, and the errors for
    tables that end before l_max."""
    from scipy.interpolate import CubicSpline
    d = str(tmp_path) + "/"
    lmax = 300
    keys = write_spectrum_files(d, lmax, step=3, lmin_tab=3)
    (tmp_path / "s.ini").write_text(f"[model]\ndirectory = {d}\nT_lmax = {lmax}\nE_lmax = 250\n"
                                    f"do_polarisation = 1\n{keys}[basis]\nuselens = 1\n")
    ini = mf.read_ini(os.fspath(tmp_path / "s.ini"))
    sp = mf.load_spectra(ini, lens=True, tl=True)
    lens = np.loadtxt(tmp_path / "lensed.txt")
    l = np.arange(lmax + 1.0)
    want = CubicSpline(lens[:, 0], lens[:, 1], bc_type="natural")(l[3:]) * 2 * np.pi / (l[3:] * (l[3:] + 1))
    assert np.all(sp["cl_tt"][:3] == 0)  # below the first tabulated l (3 - 1/2)
    assert np.max(np.abs(sp["cl_tt"][3:] - want)) <= 1e-13 * np.max(np.abs(want))
    i = 6  # a tabulated l: the spline passes through the table value
    assert abs(sp["cl_tt"][i] - 2 * np.pi * lens[1, 1] / (i * (i + 1))) <= 1e-15 * sp["cl_tt"][i]
    bn = np.loadtxt(tmp_path / "bn_t.txt")
    pix = np.loadtxt(tmp_path / "pixw.txt")[:, 1]
    wb = CubicSpline(bn[:, 0], bn[:, 1], bc_type="natural")(l[3:]) * pix[3:lmax + 1]
    assert np.max(np.abs(sp["beam_tt"][3:] - wb)) <= 1e-13
    assert sp["beam_te"].size == 251 and np.allclose(sp["beam_te"], np.sqrt(sp["beam_tt"][:251] * sp["beam_ee"]))
    assert np.all(sp["noise_te"] == 0) and sp["spec9"].shape == (9, lmax + 1)
    sc = np.loadtxt(tmp_path / "scalar.txt")
    tp = CubicSpline(sc[:, 0], sc[:, 5], bc_type="natural")(l[3:]) / l[3:] ** 3
    assert np.max(np.abs(sp["cl_tp"][3:] - tp)) <= 1e-13 * np.max(np.abs(tp))
    tl = np.loadtxt(tmp_path / "tl.txt")
    assert sp["t_wgt"][0] == 0 and abs(sp["t_wgt"][6] - tl[2, 1]) <= 1e-15
    ct = sp["cl_total"]
    assert np.allclose(ct[3:], sp["cl_tt"][3:] + sp["noise_tt"][3:] / sp["beam_tt"][3:] ** 2, rtol=1e-15, atol=0)
    (tmp_path / "t.ini").write_text(f"[model]\ndirectory = {d}\nT_lmax = 400\n{keys}")
    with pytest.raises(ValueError):  # the tables end at l = 302
        mf.load_spectra(mf.read_ini(os.fspath(tmp_path / "t.ini")))
    (tmp_path / "x.txt").write_text("# header\n1 2\n3 4 5\n")
    assert mf.load_txt_dbl(os.fspath(tmp_path / "x.txt"), 3).tolist() == [[1, 2, 0], [3, 4, 5]]


def test_basis_late_order5_uses_t_wgt_by_row(tmp_path):
    """Order 5: Fourier columns, then t_wgt (row-indexed, as the reference reads
    it), w/z, w z, t_wgt w/z and t_wgt w z."""
    import math
    (tmp_path / "b.ini").write_text("[model]\nT_lmin = 2\nT_lmax = 100\n[basis]\norder_late = 5\n")
    ini = mf.read_ini(os.fspath(tmp_path / "b.ini"))
    tw = 1.0 + np.arange(101) * 0.01
    B, _ = mf.basis_late(ini, 10, spectra={"t_wgt": tw})
    assert np.array_equal(B[:, :6], mf.basis_fourier(np.arange(2, 101.0), 5, 2.0, 100.0))
    assert B[0, 6] == tw[0] and np.all(B[0, 7:] == 0)
    i, T = 40, 42.0
    x = T * (T + 1) / (100 * 101.0)
    z, wv = math.sqrt(x), math.pow((2 * T + 1) / 201.0, 1 / 6)
    assert np.allclose(B[i, 6:], [tw[i], wv / z, wv * z, tw[i] * wv / z, tw[i] * wv * z], rtol=1e-15, atol=0)


SPEC_ROWS = ["cl_tt", "cl_te", "cl_ee", "beam_tt", "beam_te", "beam_ee", "noise_tt", "noise_te", "noise_ee", "cl_tp",
             "t_wgt"]


def _close(a, b, rtol):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin) and np.array_equal(a[~fin], b[~fin])  # l = 0 of a D_l table: inf
    scale = np.max(np.abs(b[fin])) if fin.any() else 1.0
    assert np.max(np.abs(a[fin] - b[fin]), initial=0.0) <= rtol * scale


@pytest.mark.parametrize("name", list(CASES))
def test_data_store_matches_reference(tmp_path, golden, name):
    """modal_files against the reference's own parameter.c / fixed_data.c / io.c
    compiled in place (golden, one INI case per order_late 1-10): file names,
    mode lists and pmax values identical; spectra to 1e-13 (the two natural
    splines round differently); basis tables identical for the Legendre,
    Fourier and sin-log families and their closed-form columns (1e-13 where the
    spectra enter), the 'bi' family to 1e-12; transfer files read back
    identical."""
    import json
    g = golden("files_ref")
    ol, op, pol, lens, tmin, tmax, emin, emax, terms, absolute = CASES[name]
    d = str(tmp_path) + "/"
    ini = mf.read_ini(write_case(d, name))
    # file names
    ref_names = json.loads(str(g[f"{name}_names"]))
    ours = {k: v for k, v in mf.output_names(ini).items()}
    pn = mf.proj_names(ini)
    ours.update(proj_T_data=pn["T_data"], proj_E_data=pn["E_data"], proj_T_size=pn["T_size"], proj_E_size=pn["E_size"],
                pixw=mf._ini_path(ini, "model:pixw_file", ""), BN_TT=mf._ini_path(ini, "model:BN_TT_file", ""),
                BN_EE=mf._ini_path(ini, "model:BN_EE_file", ""),
                transfer_wgt=mf._ini_path(ini, "model:transfer_wgt_file", ""))
    for k, v in ref_names.items():
        assert ours[k].replace(d, "{DIR}/") == v, (k, ours[k], v)
    # mode lists
    lo = mf.late_orders(ini, terms)
    prim, pmax_prim = mf.prim_order(ini, terms)
    assert np.array_equal(prim, g[f"{name}_prim"]) and np.array_equal(lo["ttt"], g[f"{name}_ttt"])
    for k in ("tte", "tee", "eee") if pol else ():
        assert np.array_equal(lo[k], g[f"{name}_{k}"]), k
    assert [pmax_prim, lo["pmax_T"], lo["pmax_E"]] == g[f"{name}_pmax"].tolist()
    # spectra
    sp = mf.load_spectra(ini, lens=True, tl=True)
    ref = g[f"{name}_spectra"]
    for r, k in enumerate(SPEC_ROWS):
        if k in sp:
            v = np.zeros(tmax + 1)
            v[:min(tmax + 1, sp[k].size)] = sp[k][:tmax + 1]
            _close(v, ref[r], 1e-13)
    # basis tables
    B, E = mf.basis_late(ini, lo["pmax_T"], lo["pmax_E"] if pol else None, sp)
    rb = g[f"{name}_basis_T"]
    if ol == 10:  # row 0 of columns pmax-3, pmax-2: left uninitialised by the reference
        rb = rb.copy()
        rb[0, -4:-2] = B[0, -4:-2]
    if ol in (1, 2, 3, 7):
        _close(B, rb, 1e-12)
    elif ol in (5, 6):
        _close(B, rb, 1e-13)
    else:
        assert np.array_equal(B, rb)
    if pol:
        _close(E, g[f"{name}_basis_E"], 1e-12)
    # transfer files: written by write_qtilde, read by the reference's read_qtilde and by ours
    x, qt, qe = qtilde_tables(name, pmax_prim + 1)
    mf.write_qtilde(ini, x, qt, qe if pol else None)
    q = mf.read_qtilde(ini, pmax_prim)
    assert np.array_equal(q["x"], g[f"{name}_q_x"]) and np.array_equal(q["lvec_T"], g[f"{name}_q_lvec_T"])
    assert np.array_equal(q["qt_T"], g[f"{name}_q_qt_T"].transpose(2, 0, 1))
    if pol:
        assert np.array_equal(q["qt_E"], g[f"{name}_q_qt_E"].transpose(2, 0, 1))
