"""Synthetic inputs in the reference's on-disk formats (INI file, order files,
spectrum, beam-and-noise, pixel-window and transfer-weight tables, transfer
functions), written the same way by tests/golden/make_golden.py and by the
tests that compare modal_files with the reference's data-store code run on
them."""
import os

import numpy as np

# (order_late, order_prim, do_polarisation, uselens, T_lmin, T_lmax, E_lmin, E_lmax, terms, absolute proj_file)
CASES = {
    "l1": (1, 1, 0, 1, 2, 90, 2, 90, 12, False),
    "l2": (2, 2, 1, 1, 2, 90, 3, 70, 14, False),
    "l3": (3, 3, 0, 1, 2, 90, 2, 90, 20, False),
    "l4": (4, 5, 0, 0, 2, 80, 2, 80, 16, False),
    "l5": (5, 2, 0, 1, 2, 60, 2, 60, 16, False),
    "l6": (6, 4, 1, 1, 2, 90, 3, 70, 18, False),
    "l7": (7, 3, 0, 1, 3, 75, 2, 75, 15, True),
    "l8": (8, 1, 1, 0, 2, 64, 2, 50, 12, False),
    "l9": (9, 4, 0, 1, 2, 90, 2, 90, 17, False),
    "l10": (10, 3, 0, 0, 3, 85, 2, 85, 19, True),
}


def _walk(n):
    """A case-2-like walk of sorted triples (p <= r <= s), n of them."""
    out, s = [], 0
    while len(out) < n:
        for k in range(s, -1, -1):
            for j in range(k, -1, -1):
                i = s - j - k
                if 0 <= i <= j and len(out) < n:
                    out.append((i, j, k))
        s += 1
    return np.array(out[:n], dtype=np.int64)


def write_spectrum_tables(d, lmax, step=1, lmin_tab=0):
    """Lensed and scalar cls (D_l), TT/EE beam-and-noise tables, a pixel window
    and a transfer-weight table, tabulated every `step` l from lmin_tab.
    Returns the INI lines naming them."""
    l = np.arange(lmin_tab, lmax + 5, step, dtype=np.float64)
    dl = 1e3 * np.exp(-(l / 900.0) ** 2) * (1 + 0.1 * np.sin(l / 17.0))
    lens = np.stack([l, dl, 0.05 * dl, 0.01 * dl, 0.3 * dl * np.cos(l / 9.0)], 1)
    scal = np.stack([l, dl, 0.05 * dl, 0.3 * dl, 0.2 * dl, 1e-3 * dl * (l + 1.0)], 1)
    with open(os.path.join(d, "lensed.txt"), "w") as f:
        f.write("# l TT EE BB TE\n")
        np.savetxt(f, lens)
    np.savetxt(os.path.join(d, "scalar.txt"), scal)
    np.savetxt(os.path.join(d, "bn_t.txt"), np.stack([l, np.exp(-l * l * 1e-6), 1e-5 + 0 * l], 1))
    np.savetxt(os.path.join(d, "bn_e.txt"), np.stack([l, np.exp(-l * l * 2e-6), 3e-5 + 0 * l], 1))
    lp = np.arange(0, lmax + 5, dtype=np.float64)
    np.savetxt(os.path.join(d, "pixw.txt"), np.stack([lp, 1.0 - 1e-5 * lp], 1))
    lt = np.arange(0, lmax + 5, step, dtype=np.float64)  # load_TL evaluates from l = 1
    np.savetxt(os.path.join(d, "tl.txt"), np.stack([lt, 1.0 / (1.0 + lt / 500.0)], 1))
    return ("cls_lensed_file = lensed.txt\ncls_scalar_file = scalar.txt\nBN_TT_file = bn_t.txt\n"
            "BN_EE_file = bn_e.txt\npixw_file = pixw.txt\ntransfer_wgt_file = tl.txt\n")


def write_case(d, name):
    """Write case `name` into directory d (ending in '/'); returns the INI path.
    The transfer-function files are written by the caller once pmax_prim is
    known (write_qtilde_files)."""
    ol, op, pol, lens, tmin, tmax, emin, emax, terms, absolute = CASES[name]
    raw = _walk(3 * terms + 8)
    np.savetxt(d + "ttt.txt", raw, fmt="%d")
    np.savetxt(d + "prim.txt", raw, fmt="%d")
    np.savetxt(d + "tte.txt", np.stack([raw[:, 0] % 4, raw[:, 1] % 4, raw[:, 2] % 3], 1), fmt="%d")
    np.savetxt(d + "tee.txt", np.stack([raw[:, 1] % 3, raw[:, 2] % 3, raw[:, 0] % 5], 1), fmt="%d")
    np.savetxt(d + "eee.txt", raw % 4, fmt="%d")
    keys = write_spectrum_tables(d, max(tmax, emax), step=2)
    proj = (d + "tr") if absolute else "proj"
    ini = (f"; synthetic case {name}\n[model]\ndirectory = \"{d}\"\nT_lmin = {tmin}\nT_lmax = {tmax}\n"
           f"E_lmin = {emin}\nE_lmax = {emax}\ndo_polarisation = {pol}\ndelta_phi = 0.5\nfskyT = 0.8\nfskyE = 0.6\n"
           f"order_TTT_file_late = ttt.txt\norder_TTE_file_late = tte.txt\norder_TEE_file_late = tee.txt\n"
           f"order_EEE_file_late = eee.txt   ; the EEE list\norder_file_prim = prim.txt\n{keys}"
           f"[basis]\nterms = {terms}\norder_late = {ol}\norder_prim = {op}\nuselens = {lens}\nproj_file = {proj}\n"
           f"do3D = 1\n[old]\ngflag_pca = 1\n")
    path = d + "run.ini"
    with open(path, "w") as f:
        f.write(ini)
    return path


def qtilde_tables(name, P, xsize=7):
    """Transfer functions [xsize][P][lsize] and x grid for case `name`: l rows
    0..T_lmax (+3, so the files hold more rows than the drivers use)."""
    tmax, emax = CASES[name][5], CASES[name][7]
    L = max(tmax, emax) + 4
    x = np.linspace(100.0, 900.0, xsize)
    l = np.arange(L, dtype=np.float64)
    p = np.arange(P)[:, None]
    qt = np.stack([np.cos((p + 1) * xi / 400.0) * np.sin(0.05 * l * (1 + p)) / (1.0 + l) for xi in x])
    return x, qt, 0.5 * qt + 0.01
