"""Reference-compatible file formats and INI-driven drivers for the GPU path.

The reference's drivers read an iniparser INI file (parameter.c:127-980), name
their outputs from its keys (parameter.c:243-700), and write raw native FP64
arrays (array_write / array_read, arrays.c:6-77).  This module restates those
conventions so that results of the GPU path land in the files the reference's
later stages read:

  read_ini(path)                     -> {"section:key": "value"} (iniparser keys)
  output_names(ini)                  -> the orthol/lambdal/modes/gamma file names
  array_write(path, a) / array_read  -> raw native FP64, no header
  load_three_int(path)               -> [n][3] mode orderings (io.c:229-257)
  load_spectra(ini, ...)             -> load_cl / load_BN / load_lens / load_TL on integer l
  late_orders(ini, N)                -> set_terms_late orderings 1 to 10 (TTT and polarised)
  basis_late(ini, pmax_t, ...)       -> create_basis_late's basis tables (orders 1-10)
  prim_order(ini, N)                 -> set_terms_prim orderings 1 to 5 and pmax_prim
  proj_names(ini)                    -> the proj_T/E data and size file names
  read_qtilde / write_qtilde         -> the transfer-function files (read_qtilde,
                                        output_qtilde, fixed_data.c:2076-2435)
  ortho_late(ini_path, basis_t, ...) -> ortho_late_mpi.c's outputs from the GPU
  gamma_late(ini_path, basis_t, ...) -> gamma_mpi.c's gamma_XXX files from the GPU
  modes_late(ini_path, basis_t, ...) -> eigenmodetoday_mpi.c's modes_TTT_<model> files
  prune_late(ini_path, ...)          -> basis_optimisation_mpi.c's elimination order, printed

Command line:
  python modal_files.py ortho_late <ini> [<basis_T.unf> --pt P] [--basis-e <basis_E.unf> --pe PE] [--split]
  python modal_files.py gamma_late <ini> [<basis_T.unf> --pt P] [--cl <cl_total.unf>]
      [--basis-e <basis_E.unf> --pe PE --spec9 <spec9.unf>]
  python modal_files.py modes_late <ini> [<basis_T.unf> --pt P] [--cl <cl_total.unf>] --tab <shape.npy> --model M
  python modal_files.py prune_late <ini> [--gamma <gamma.unf>] [--faillist <faillist.txt>]
Mode lists come from the INI file as set_terms_late builds them.  Basis files
are raw FP64 [L][P] tables (basis_late_T / basis_late_E layouts,
fixed_data.c:1764); without one the drivers build create_basis_late's table;
the spectra come from the INI's cls / BN / pixel-window files (load_spectra),
or as raw FP64: cl_total over l = 0..T_lmax (C_l + N_l/b_l^2 of the TT
weight) and spec9 [9][T_lmax+1] (cl TT, TE, EE, beam TT, TE, EE, noise TT,
TE, EE).
"""
import argparse
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


# ------------------------------------------------------------------ INI

def read_ini(path):
    """iniparser-style dictionary: keys 'section:key' in lower case, values
    with surrounding quotes removed; ';' and '#' start comment lines and end
    unquoted values."""
    out, section = {}, ""
    with open(path) as f:
        for raw in f:
            line = raw.strip()
            if not line or line[0] in ";#":
                continue
            m = re.match(r"^\[(.*)\]$", line)
            if m:
                section = m.group(1).strip().lower()
                continue
            if "=" not in line:
                continue
            key, val = line.split("=", 1)
            val = val.strip()
            if val[:1] and val[:1] in "\"'":
                q = val[0]
                end = val.find(q, 1)
                val = val[1:end] if end > 0 else val[1:]
            else:
                val = re.split(r"[;#]", val, maxsplit=1)[0].strip()
            out[f"{section}:{key.strip().lower()}"] = val
    return out


def _strtol0(v):
    """C strtol(v, NULL, 0): optional sign, 0x hex, leading-0 octal, else
    decimal, up to the first character that does not fit (0 if none)."""
    m = re.match(r"\s*([+-]?)(0[xX][0-9a-fA-F]+|0[0-7]*|[1-9][0-9]*)", v)
    if not m:
        return 0
    digits = m.group(2)
    base = 16 if digits[:2] in ("0x", "0X") else (8 if digits.startswith("0") and len(digits) > 1 else 10)
    n = int(digits, base)
    return -n if m.group(1) == "-" else n


def _atof(v):
    """C atof: the longest decimal floating-point prefix (0.0 if none)."""
    m = re.match(r"\s*[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?", v)
    return float(m.group(0)) if m else 0.0


def _get(ini, key, default, conv=str):
    v = ini.get(key.lower())
    if v is None:
        return default
    try:
        return conv(v)
    except ValueError:
        return default


def getint(ini, key, default):
    """iniparser_getint: strtol(value, NULL, 0)."""
    return _get(ini, key, default, _strtol0)


def getdouble(ini, key, default):
    """iniparser_getdouble: atof(value)."""
    return _get(ini, key, default, _atof)


def getstring(ini, key, default):
    return _get(ini, key, default, str)


# ------------------------------------------------------------ file names

def _params(ini):
    return dict(directory=getstring(ini, "model:directory", ""), T_lmax=getint(ini, "model:T_lmax", 1000),
                E_lmax=getint(ini, "model:E_lmax", 1000), T_lmin=getint(ini, "model:T_lmin", 2),
                E_lmin=getint(ini, "model:E_lmin", 2), terms=getint(ini, "basis:terms", 101),
                order_prim=getint(ini, "basis:order_prim", 3), order_late=getint(ini, "basis:order_late", 3),
                do_polarisation=getint(ini, "model:do_polarisation", 0), gflag_pca=getint(ini, "old:gflag_pca", 1))


def output_names(ini):
    """File names of parameter.c for the late-time products: orthol_XXX,
    lambdal_XXX, modes_XXX and gamma_XXX (XXX = TTT, TTE, TEE, EEE).  A value
    starting with '/' is taken as it is (only for TTT, as the reference)."""
    p = _params(ini)
    s1, s2, s3, s4, s5 = (str(p[k]) for k in ("T_lmax", "E_lmax", "terms", "order_prim", "order_late"))
    s6, s7 = str(p["T_lmin"]), str(p["E_lmin"])
    T, E = f"{s6}-{s1}", f"{s7}-{s2}"
    ranges = {"TTT": T, "TTE": f"{T}_{E}", "TEE": f"{T}_{E}", "EEE": E}
    names = {}
    for fam, key, default, mid in [("orthol", "basis:orthol_file", "orthol", [s5, s3]),
                                   ("lambdal", "basis:lambdal_file", "lambdal", [s5, s3]),
                                   ("modes", "basis:modes_file", "modes", [s5, s3]),
                                   ("gamma", "basis:gamma_file", "gamma", [s4, s5, s3])]:
        v = getstring(ini, key, default)
        for x in ("TTT", "TTE", "TEE", "EEE"):
            if v.startswith("/"):
                if fam == "gamma":
                    names[f"{fam}_{x}"] = f"{v}_{x}"  # parameter.c:638-645
                elif x == "TTT":
                    names[f"{fam}_{x}"] = v
                continue
            names[f"{fam}_{x}"] = p["directory"] + v + f"_{x}_" + ranges[x] + "_" + "_".join(mid)
    return names


# ------------------------------------------------------------ raw arrays

def array_write(path, a):
    """array_write (arrays.c:6-21): the doubles of a, native order, no header."""
    np.ascontiguousarray(a, dtype=np.float64).tofile(path)


def array_read(path, n=None):
    """array_read (arrays.c:56-77): n doubles (all when n is None)."""
    a = np.fromfile(path, dtype=np.float64)
    if n is not None:
        if a.size < n:
            raise ValueError(f"{path}: {a.size} doubles, {n} expected")
        a = a[:n]
    return a


def load_three_int(path):
    """load_three_int (io.c:229-257): whitespace-separated integer triples."""
    v = np.loadtxt(path, dtype=np.int64, ndmin=2)
    return v.reshape(-1, 3).astype(np.int32)


# ------------------------------------------------------------ mode orders

def _order_case1(N):
    out, i, j, k, s = [], 0, 0, 0, 0
    for _ in range(N):  # set_terms_late case 1 (fixed_data.c:305-321)
        out.append((i, j, k))
        if k - j < 2 and j - i < 2 and k - i < 2:
            s += 1
            i = j = 0
            k = s
        elif k - j > 1:
            k -= 1
            j += 1
        else:
            i += 1
            j = i
            k = s - 2 * i
    return np.array(out, dtype=np.int32)


def _order_case2(N):
    out, i, j, k, s = [], 0, 0, 0, 0
    for _ in range(N):  # set_terms_late case 2 (fixed_data.c:362-378)
        out.append((i, j, k))
        if i < j:
            j -= 1
            k += 1
        elif i > 0:
            i -= 1
            j = (s - i) // 2
            k = s - j - i
        else:
            s += 1
            i = s // 3
            j = (s - i) // 2
            k = s - i - j
    return np.array(out, dtype=np.int32)


# set_terms_late (fixed_data.c:272-953): orders 4-7, 9 and 10 read the TTT
# file shifted down by SHIFT places and put special triples (offsets from the
# pre-insertion pmax_T) in the freed rows; pmax_T then grows by PMAX_ADD.
_LATE_SHIFT = {3: 0, 4: 1, 5: 3, 6: 4, 7: 1, 8: 0, 9: 1, 10: 3}
_LATE_SPECIAL = {
    4: [(1, (1, 1, 2))],
    5: [(1, (1, 1, 1)), (2, (2, 2, 3)), (3, (4, 4, 5))],
    6: [(1, (1, 1, 2)), (2, (3, 5, 8)), (3, (3, 6, 7)), (4, (4, 5, 6))],
    7: [(1, (1, 1, 2))],
    9: [(1, (1, 1, 2))],
    10: [(0, (2, 2, 4)), (1, (1, 3, 4)), (2, (1, 1, 5))],
}
_LATE_PMAX_ADD = {4: 2, 5: 5, 6: 8, 7: 2, 9: 2, 10: 5}


def _order_file(ini, key, default, N, what):
    p = _params(ini)
    f = getstring(ini, key, default)
    path = f if f.startswith("/") else p["directory"] + f
    t = load_three_int(path)
    if t.shape[0] < N:
        raise ValueError(f"eigenfunction {N} exceeds that in {what} distance file {path}")
    return t


def late_orders(ini, N, pol=None, pol_lists=None):
    """set_terms_late (fixed_data.c:272-953) for basis:order_late 1 to 10:
    {"ttt", "tte", "tee", "eee" (with model:do_polarisation 1), "pmax_T",
    "pmax_E"}.  Orders 1 and 2 walk the triples; the others read
    model:order_TTT_file_late, orders 4-7, 9 and 10 shifted down with their
    extra-function triples put in (the basis columns create_basis_late appends
    for them).  The polarised lists come from the TTE/TEE/EEE files; a TEE file
    line (a, b, c) is the triple (c, a, b), T index first.  pmax_T and pmax_E
    are the largest indices as the reference counts them (third entries, and
    the T/E entries of the polarised lists).  pol (default: do_polarisation
    is 1) switches the polarised lists on; pol_lists = (tte, tee, eee), T
    indices first, stands in for their files.  A file shorter than N raises
    ValueError (the reference prints a message and goes on)."""
    case = getint(ini, "basis:order_late", 3)
    if case == 1:
        ttt = _order_case1(N)
    elif case == 2:
        ttt = _order_case2(N)
    elif case in _LATE_SHIFT:
        raw = _order_file(ini, "model:order_TTT_file_late", "order_dist.txt", N, "TTT")
        k = _LATE_SHIFT[case]
        ttt = raw[:N].copy()
        if k:
            # rows above the shift hold the file's rows k places earlier (row 0..k unchanged,
            # as the reference's in-place downward copy leaves them; order 10 also moves row k)
            start = k if case == 10 else k + 1
            ttt[start:] = raw[start - k:N - k]
    else:
        raise ValueError(f"invalid mode {case} specified for eigen function ordering")
    out = {"ttt": np.ascontiguousarray(ttt, dtype=np.int32)}
    pmax_t, pmax_e = int(ttt[:, 2].max()), 0
    if _params(ini)["do_polarisation"] == 1 if pol is None else pol:
        if pol_lists is None:
            tte = _order_file(ini, "model:order_TTE_file_late", "order_dist_XXY.txt", N, "TTE")[:N]
            tee = _order_file(ini, "model:order_TEE_file_late", "order_dist_XXY.txt", N, "TEE")[:N][:, [2, 0, 1]]
            eee = _order_file(ini, "model:order_EEE_file_late", "order_dist.txt", N, "EEE")[:N]
        else:
            tte, tee, eee = (np.asarray(o, dtype=np.int32).reshape(-1, 3)[:N] for o in pol_lists)
        pmax_t = max(pmax_t, int(tte[:, 1].max()), int(tee[:, 0].max()))
        pmax_e = max(int(tte[:, 2].max()), int(tee[:, 2].max()), int(eee[:, 2].max()))
        out.update(tte=np.ascontiguousarray(tte, dtype=np.int32), tee=np.ascontiguousarray(tee, dtype=np.int32),
                   eee=np.ascontiguousarray(eee, dtype=np.int32))
    for row, offs in _LATE_SPECIAL.get(case, []):
        if row < N:
            out["ttt"][row] = [pmax_t + o for o in offs]
    out["pmax_T"] = pmax_t + _LATE_PMAX_ADD.get(case, 0)
    out["pmax_E"] = pmax_e
    return out


def mode_order(ini, N):
    """The TTT mode triples of set_terms_late without the polarised lists
    (late_orders(ini, N, pol=False)["ttt"]; with polarisation the extra-function
    triples of orders 4-7, 9 and 10 also count the polarised T indices)."""
    return late_orders(ini, N, pol=False)["ttt"]


# ------------------------------------------------------------ spectra

def _ini_path(ini, key, default):
    """A file key of parameter.c: absolute as given, else directory + value."""
    v = getstring(ini, key, default)
    return v if v.startswith("/") else _params(ini)["directory"] + v


def load_txt_dbl(path, columns):
    """load_txt_dbl (io.c:64-93): lines starting with '#' skipped, the first
    `columns` numbers of every other line (missing ones read as 0).  Returns
    [rows][columns]."""
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                continue
            vals = []
            for tok in line.split()[:columns]:
                try:
                    vals.append(float(tok))
                except ValueError:
                    break
            rows.append(vals + [0.0] * (columns - len(vals)))
    return np.array(rows, dtype=np.float64).reshape(-1, columns)


def natural_spline(x, y):
    """Natural cubic spline through (x, y) (zero second derivative at both
    ends), the interpolant of GSL's gsl_interp_cspline that load_cl / load_BN
    use.  Restated from its definition: the second derivatives M solve
    h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1}
      = 6 ((y_{i+1} - y_i)/h_i - (y_i - y_{i-1})/h_{i-1}).
    Returns f(t) for t in [x_0, x_last]; outside it raises ValueError (GSL
    stops there with a domain error)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = x.size
    if n < 3 or np.any(np.diff(x) <= 0):
        raise ValueError("a natural spline needs at least 3 increasing abscissae")
    h = np.diff(x)
    M = np.zeros(n)
    if n > 2:
        diag = 2.0 * (h[:-1] + h[1:])
        off = h[1:-1].copy()
        rhs = 6.0 * (np.diff(y[1:]) / h[1:] - np.diff(y[:-1]) / h[:-1])
        m = n - 2
        cp, dp = np.zeros(m), np.zeros(m)  # Thomas algorithm on the symmetric tridiagonal system
        for i in range(m):
            den = diag[i] - (off[i - 1] * cp[i - 1] if i else 0.0)
            cp[i] = off[i] / den if i < m - 1 else 0.0
            dp[i] = (rhs[i] - (off[i - 1] * dp[i - 1] if i else 0.0)) / den
        for i in range(m - 1, -1, -1):
            M[i + 1] = dp[i] - (cp[i] * M[i + 2] if i < m - 1 else 0.0)

    def f(t):
        t = np.asarray(t, dtype=np.float64)
        if np.any(t < x[0]) or np.any(t > x[-1]):
            raise ValueError(f"spline evaluated outside [{x[0]}, {x[-1]}]")
        i = np.clip(np.searchsorted(x, t, side="right") - 1, 0, n - 2)
        hi, a, b = h[i], x[i + 1] - t, t - x[i]
        return (M[i] * a ** 3 + M[i + 1] * b ** 3) / (6.0 * hi) + (y[i] / hi - M[i] * hi / 6.0) * a \
            + (y[i + 1] / hi - M[i + 1] * hi / 6.0) * b
    return f


def _on_l(lmax, l_raw, y_raw, scale=None):
    """Spline of a table onto l = 0..lmax, zero for l <= l_raw[0] - 1/2 (the
    reference's guard), with scale(l) applied to the interpolated value."""
    out = np.zeros(lmax + 1)
    l = np.arange(lmax + 1, dtype=np.float64)
    on = l > l_raw[0] - 0.5
    if np.any(on):
        v = natural_spline(l_raw, y_raw)(l[on])
        with np.errstate(divide="ignore", invalid="ignore"):  # l = 0 in a D_l table gives inf, as in C
            out[on] = v if scale is None else scale(l[on], v)
    return out


def load_spectra(ini, lens=False, tl=False):
    """load_cl, load_BN, load_lens and load_TL (fixed_data.c:1116-1498, 1542-1597):
    spectra on integer l from the INI file's tables, by natural cubic splines.
      cl_tt (and cl_te, cl_ee with do_polarisation) over l = 0..T_lmax
        (E_lmax), 2 pi D_l / (l (l+1)) from model:cls_lensed_file (l, TT, EE,
        BB, TE) with basis:uselens 1, else model:cls_scalar_file (l, TT, EE,
        TE, P, PT);
      beam_tt = pixel window x spline of model:BN_TT_file (l, beam, noise),
        noise_tt = spline of its noise; the pixel window (model:pixw_file,
        l, w) is taken by row index, as the reference does; E likewise from
        model:BN_EE_file; beam_te = sqrt(beam_tt beam_ee), noise_te = 0;
      cl_tp (lens): spline of the scalar file's PT column / l^3;
      t_wgt (tl): spline of model:transfer_wgt_file (l, T_l) at l = 1..T_lmax.
    Values at l <= (first tabulated l) - 1/2 are 0, as the reference sets them.
    Also cl_total = cl_tt + noise_tt / beam_tt^2 at l >= 2 (the TT weight's
    spectrum, 1 below l = 2), and spec9 for the polarised transfer Gamma."""
    import math
    p = _params(ini)
    lT, lE = p["T_lmax"], p["E_lmax"]
    pol = p["do_polarisation"] == 1
    out = {}
    dl2cl = lambda l, v: 2.0 * math.pi * v / (l * (l + 1.0))  # noqa: E731
    if getint(ini, "basis:uselens", 1) == 1:
        d = load_txt_dbl(_ini_path(ini, "model:cls_lensed_file", "cls_planck_DDX9_lensed.txt"), 5)
        cols = {"tt": 1, "ee": 2, "te": 4}
    else:
        d = load_txt_dbl(_ini_path(ini, "model:cls_scalar_file", "cls_planck_DDX9_scalar.txt"), 6)
        cols = {"tt": 1, "ee": 2, "te": 3}
    if lT > d[-1, 0]:
        raise ValueError(f"Cls do not contain enough l's, max data {lT} max cl: {int(d[-1, 0])}")
    out["cl_tt"] = _on_l(lT, d[:, 0], d[:, cols["tt"]], dl2cl)
    if pol:
        out["cl_te"] = _on_l(lE, d[:, 0], d[:, cols["te"]], dl2cl)
        out["cl_ee"] = _on_l(lE, d[:, 0], d[:, cols["ee"]], dl2cl)
    pix = load_txt_dbl(_ini_path(ini, "model:pixw_file", "pixwgt_2048.txt"), 2)[:, 1]
    for x, lm in (("tt", lT),) + ((("ee", lE),) if pol else ()):
        bn = load_txt_dbl(_ini_path(ini, f"model:BN_{x.upper()}_file", f"BN_{x.upper()}.txt"), 3)
        if lm > bn[-1, 0]:
            raise ValueError(f"BN {x.upper()} do not contain enough l's, max data {lm} max BN: {int(bn[-1, 0])}")
        if pix.size < lm + 1:
            raise ValueError(f"pixel window has {pix.size} rows, l = 0..{lm} needs {lm + 1}")
        out[f"beam_{x}"] = _on_l(lm, bn[:, 0], bn[:, 1], lambda l, v: pix[l.astype(np.int64)] * v)
        out[f"noise_{x}"] = _on_l(lm, bn[:, 0], bn[:, 2])
    if pol:
        out["beam_te"] = np.sqrt(out["beam_tt"][:lE + 1] * out["beam_ee"])
        out["noise_te"] = np.zeros(lE + 1)
    if lens:
        d6 = load_txt_dbl(_ini_path(ini, "model:cls_scalar_file", "cls_planck_DDX9_scalar.txt"), 6)
        if lT > d6[-1, 0]:
            raise ValueError(f"Cls do not contain enough l's, max data {lT} max cl: {int(d6[-1, 0])}")
        out["cl_tp"] = _on_l(lT, d6[:, 0], d6[:, 5], lambda l, v: v / (l * l * l))
    if tl:
        t = load_txt_dbl(_ini_path(ini, "model:transfer_wgt_file", "wmap7_Tl.txt"), 2)
        if lT > t[-1, 0]:
            raise ValueError(f"T do not contain enough l's, max data {lT} max T: {int(t[-1, 0])}")
        w = np.zeros(lT + 1)
        w[1:] = natural_spline(t[:, 0], t[:, 1])(np.arange(1, lT + 1, dtype=np.float64))
        out["t_wgt"] = w
    ct = np.ones(lT + 1)
    with np.errstate(divide="ignore", invalid="ignore"):  # zero beam below the tables: not finite, rejected later
        ct[2:] = out["cl_tt"][2:] + out["noise_tt"][2:] / (out["beam_tt"][2:] * out["beam_tt"][2:])
    out["cl_total"] = ct
    if pol:
        n = lT + 1

        def ext(a):
            e = np.zeros(n)
            e[:min(n, a.size)] = a[:n]
            return e
        out["spec9"] = np.stack([out["cl_tt"], ext(out["cl_te"]), ext(out["cl_ee"]), out["beam_tt"],
                                 ext(out["beam_te"]), ext(out["beam_ee"]), out["noise_tt"], ext(out["noise_te"]),
                                 ext(out["noise_ee"])])
    return out


# ------------------------------------------------------------ basis tables

def _libm(f, a):
    """Elementwise libm call (math module), so that values match C's cos/sin/
    log/pow bit for bit."""
    return np.frompyfunc(f, 1, 1)(a).astype(np.float64)


def basis_fourier(values, pmax, vmin, vmax):
    """basis_functions_fourier (basis_functions.c:6-27): column j is
    cos(pi n x) for even j and sin(pi n x) for odd j, n = j + j%2,
    x = (v - min)/(max - min)."""
    import math
    x = (np.asarray(values, dtype=np.float64) - vmin) / (vmax - vmin)
    out = np.empty((x.size, pmax + 1))
    for j in range(pmax + 1):
        k = j % 2
        arg = (math.pi * (j + k)) * x
        out[:, j] = _libm(math.sin if k else math.cos, arg)
    return out


def basis_sinlog(values, pmax, vmin, vmax):
    """basis_functions_sinlog (basis_functions.c:29-63): the Fourier family in
    x = log(v/min)/log(max/min); values below 1e-6 give 1 (cosines), 0 (sines)."""
    import math
    v = np.asarray(values, dtype=np.float64)
    y = 1.0 / math.log(vmax / vmin)
    small = v < 1e-6
    x = _libm(math.log, np.where(small, 1.0, v) / vmin) * y
    out = np.empty((v.size, pmax + 1))
    for j in range(pmax + 1):
        k = j % 2
        col = _libm(math.sin if k else math.cos, (math.pi * (j + k)) * x)
        out[:, j] = np.where(small, 0.0 if k else 1.0, col)
    return out


def basis_legendre(values, pmax, vmin, vmax):
    """basis_functions_legendre (basis_functions.c:88-107): shifted Legendre
    polynomials by the upward three-term recurrence, in the reference's order
    of operations."""
    x = (np.asarray(values, dtype=np.float64) - vmin) / (vmax - vmin)
    out = np.empty((x.size, pmax + 1))
    out[:, 0] = 1.0
    if pmax > 0:
        out[:, 1] = 2.0 * x - 1.0
    for j in range(2, pmax + 1):
        out[:, j] = ((2.0 * j - 1.0) * out[:, 1] * out[:, j - 1] - (j - 1.0) * out[:, j - 2]) / (1.0 * j)
    return out


def _bi_recurrence(n):
    """Recurrence coefficients (a_j, sqrt(b_j)) of the polynomials orthonormal
    on [0, 1] under the weight w(x) = 2x - 3x^2/2 (the area of the tetrapyd's
    cross-section at l1/lmax = x; integral 1/2), from exact rational moments
    m_k = 2/(k+2) - 3/(2(k+3)) by the Stieltjes procedure."""
    from fractions import Fraction as Fr
    m = [Fr(2, k + 2) - Fr(3, 2 * (k + 3)) for k in range(2 * n + 2)]

    def ip(p, q):
        return sum(pi * qk * m[i + k] for i, pi in enumerate(p) if pi for k, qk in enumerate(q) if qk)

    a, b = [], [ip([Fr(1)], [Fr(1)])]
    prev, cur = None, [Fr(1)]
    for j in range(n):
        h = ip(cur, cur)
        xc = [Fr(0)] + cur
        a.append(ip(xc, cur) / h)
        nxt = [c - (a[-1] * cur[i] if i < len(cur) else 0) for i, c in enumerate(xc)]
        if prev is not None:
            nxt = [c - (b[-1] * prev[i] if i < len(prev) else 0) for i, c in enumerate(nxt)]
        b.append(ip(nxt, nxt) / h)
        prev, cur = cur, nxt
    return [float(v) for v in a], [math_sqrt_fraction(v) for v in b]


def math_sqrt_fraction(f):
    """sqrt of a positive Fraction, correctly rounded to FP64."""
    from decimal import Decimal, getcontext
    getcontext().prec = 60
    return float((Decimal(f.numerator) / Decimal(f.denominator)).sqrt())


_BI = {}


def basis_bi(values, pmax, vmin, vmax):
    """The 'bi' family of basis_functions_bi (basis_functions.c:164-208):
    polynomials orthonormal on x = (v - min)/(max - min) in [0, 1] under the
    weight 2x - 3x^2/2, leading coefficient positive (p_0 = sqrt 2).  Restated
    from that definition and evaluated by the stable three-term recurrence;
    the reference evaluates a table of monomial coefficients (up to 1e22 at
    degree 30) by Horner's rule.  The two agree to about 1e-13 relative up to
    degree 8; above that the reference's own rounding (about 1e-16 times the
    coefficient sizes) dominates the difference."""
    if pmax not in _BI:
        _BI[pmax] = _bi_recurrence(pmax + 1)
    a, sb = _BI[pmax]
    x = (np.asarray(values, dtype=np.float64) - vmin) / (vmax - vmin)
    out = np.empty((x.size, pmax + 1))
    out[:, 0] = 1.0 / sb[0]
    prev = np.zeros_like(x)
    for j in range(pmax):
        nxt = ((x - a[j]) * out[:, j] - (sb[j] * prev if j else 0.0)) / sb[j + 1]
        prev = out[:, j]
        out[:, j + 1] = nxt
    return out


def basis_late(ini, pmax_t, pmax_e=None, spectra=None, pol=None):
    """create_basis_late (fixed_data.c:1754-1986): (basis_T [T_size][pmax_T+1],
    basis_E [E_size][pmax_E+1] or None) on l = T_lmin..T_lmax (E_lmin..E_lmax)
    for basis:order_late 1-10.  Orders 1-3 and 7 use the 'bi' polynomials
    (basis_bi), 4-6 Fourier, 8 sin-log, 9 and 10 shifted Legendre; 4-7, 9
    and 10 append their closed-form columns in
    w = ((2l+1)/(2lmax+1))^{1/6} and z = sqrt(l(l+1)/(lmax(lmax+1))), and
    order 6 those scaled by c = w/sqrt(C_l + N_l/b_l^2) with C_l and the
    lensing cross-spectrum C_l^{TP}: spectra = {"cl_tt", "noise_tt",
    "beam_tt", "cl_tp"} over l = 0..T_lmax, order 5 the transfer weight
    spectra["t_wgt"] (load_TL), taken by row index as the reference takes
    it.  load_spectra reads both from the INI's files.  Row 0 of order 10's
    columns pmax-3 and pmax-2 is
    left uninitialised by the reference; it is 0 here.  The E basis
    (model:do_polarisation 1) is bi for orders < 4 and 7, Fourier for 4-6,
    sin-log for 8 and Legendre for 9 and 10; pol overrides do_polarisation."""
    import math
    p = _params(ini)
    case = p["order_late"]
    Tmin, Tmax = float(p["T_lmin"]), float(p["T_lmax"])
    Tvec = np.arange(p["T_lmin"], p["T_lmax"] + 1, dtype=np.float64)
    n = pmax_t
    B = np.zeros((Tvec.size, n + 1))
    x = Tvec * (Tvec + 1.0) / (Tmax * (Tmax + 1.0))
    y = (2.0 * Tvec + 1.0) / (2.0 * Tmax + 1.0)
    z = np.sqrt(x)
    w = _libm(lambda v: math.pow(v, 1.0 / 6.0), y)
    if case < 4:
        B[:] = basis_bi(Tvec, n, Tmin, Tmax)
    elif case in (4, 7, 9):
        fam = {4: basis_fourier, 7: basis_bi, 9: basis_legendre}[case]
        B[:, :n - 1] = fam(Tvec, n - 2, Tmin, Tmax)
        r = slice(0 if case == 9 else 1, None)  # order 9 fills row 0 too
        B[r, n - 1] = w[r] / z[r]
        B[r, n] = w[r] * z[r]
    elif case == 6:
        if spectra is None:
            raise ValueError("order_late 6 needs cl_tt, noise_tt, beam_tt and cl_tp")
        B[:, :n - 7] = basis_fourier(Tvec, n - 8, Tmin, Tmax)
        l = np.arange(1, Tvec.size) + int(Tmin)  # the reference's l = i + Tmin for row i
        cl_tt = np.asarray(spectra["cl_tt"], dtype=np.float64)[l]
        cl_tp = np.asarray(spectra["cl_tp"], dtype=np.float64)[l]
        bt = np.asarray(spectra["beam_tt"], dtype=np.float64)[l]
        c = np.sqrt(cl_tt + np.asarray(spectra["noise_tt"], dtype=np.float64)[l] / (bt * bt))
        c = np.where(c != 0.0, w[1:] / np.where(c != 0.0, c, 1.0), c)
        xs, zs, ws = x[1:], z[1:], w[1:]
        B[1:, n - 7] = ws / zs
        B[1:, n - 6] = ws * zs
        B[1:, n - 5] = c
        B[1:, n - 4] = c * xs
        B[1:, n - 3] = c * cl_tt
        B[1:, n - 2] = c * cl_tp
        B[1:, n - 1] = c * xs * cl_tt
        B[1:, n] = c * xs * cl_tp
    elif case == 8:
        B[:] = basis_sinlog(Tvec, n, Tmin, Tmax)
    elif case == 10:
        B[:, :n - 3] = basis_legendre(Tvec, n - 4, Tmin, Tmax)
        l1 = Tvec[1:] / Tmax
        xs, zs, ws = x[1:], z[1:], w[1:]
        B[1:, n - 4] = ws / (l1 * zs)
        B[1:, n - 3] = ws / zs
        B[1:, n - 2] = ws * l1 / zs
        B[1:, n - 1] = ws * zs
        B[1:, n] = ws * (l1 * l1) * zs
    elif case == 5:
        if spectra is None or "t_wgt" not in spectra:
            raise ValueError("order_late 5 needs load_TL's t_wgt (load_spectra(ini, tl=True))")
        tw = np.asarray(spectra["t_wgt"], dtype=np.float64)
        if tw.size < Tvec.size:
            raise ValueError(f"t_wgt has {tw.size} values, {Tvec.size} rows need as many")
        tw = tw[:Tvec.size]  # by row index, as the reference reads it
        B[:, :n - 4] = basis_fourier(Tvec, n - 5, Tmin, Tmax)
        B[0, n - 4] = tw[0]
        xs, zs, ws, ts = x[1:], z[1:], w[1:], tw[1:]
        B[1:, n - 4] = ts
        B[1:, n - 3] = ws / zs
        B[1:, n - 2] = ws * zs
        B[1:, n - 1] = ts * ws / zs
        B[1:, n] = ts * ws * zs
    else:
        raise ValueError(f"invalid order_late {case}")
    E = None
    if p["do_polarisation"] == 1 if pol is None else pol:
        if pmax_e is None:
            raise ValueError("do_polarisation needs pmax_E")
        Evec = np.arange(p["E_lmin"], p["E_lmax"] + 1, dtype=np.float64)
        fam = (basis_bi if case < 4 or case == 7 else basis_fourier if case in (4, 5, 6)
               else basis_sinlog if case == 8 else basis_legendre)
        E = fam(Evec, pmax_e, float(p["E_lmin"]), float(p["E_lmax"]))
    return B, E


def prim_order(ini, N):
    """(prim[N][3], pmax_prim) of set_terms_prim (fixed_data.c:104-238) for
    basis:order_prim 1 and 2 (the same walks as set_terms_late's), 3 and 5 (the
    first N triples of model:order_file_prim) and 4 (N - 1 triples of that file
    with (pmax + 1, pmax + 1, pmax + 2) put in at index 1: the two extra
    functions whose transfer files end in _l1 and _l2).  pmax_prim is the
    largest third index.  A file shorter than N raises ValueError (the
    reference prints a message and goes on)."""
    case = getint(ini, "basis:order_prim", 3)
    if case == 1:
        t = _order_case1(N)
    elif case == 2:
        t = _order_case2(N)
    elif case in (3, 4, 5):
        p = _params(ini)
        f = getstring(ini, "model:order_file_prim", "order_dist.txt")
        path = f if f.startswith("/") else p["directory"] + f
        raw = load_three_int(path)
        if raw.shape[0] < N:
            raise ValueError(f"eigenfunction {N} exceeds that in distance file {path}")
        if case == 4:
            head = raw[:N - 1]
            pm = int(head[:, 2].max()) if N > 1 else 0
            t = np.concatenate([head[:1], np.array([[pm + 1, pm + 1, pm + 2]], dtype=np.int32), head[1:]])[:N]
        else:
            t = raw[:N]
    else:
        raise ValueError(f"invalid mode {case} specified for eigen function ordering")
    return np.ascontiguousarray(t, dtype=np.int32), int(t[:, 2].max())


# ------------------------------------------------------------ transfer files

def proj_names(ini):
    """proj_T/E data and size file names of parameter.c:725-760: directory +
    proj_file + _T_<T_lmax>_<order_prim> (data, one file per primordial index
    with _<n> appended) and _T_<T_lmax>_size; a value starting with '/' gives
    <value>_T and <value>_T_size (E likewise with E_lmax)."""
    p = _params(ini)
    v = getstring(ini, "basis:proj_file", "proj")
    if v.startswith("/"):
        return {"T_data": v + "_T", "E_data": v + "_E", "T_size": v + "_T_size", "E_size": v + "_E_size"}
    base = p["directory"] + v
    return {"T_data": f"{base}_T_{p['T_lmax']}_{p['order_prim']}", "E_data": f"{base}_E_{p['E_lmax']}_{p['order_prim']}",
            "T_size": f"{base}_T_{p['T_lmax']}_size", "E_size": f"{base}_E_{p['E_lmax']}_size"}


def _qtilde_suffixes(order_prim, pmax):
    """File suffix of each primordial index: _0 .. _pmax, or with order_prim 4
    _0 .. _(pmax-2) then _l1 and _l2 (read_qtilde, fixed_data.c:2252-2330)."""
    if order_prim != 4:
        return [str(n) for n in range(pmax + 1)]
    return [str(n) for n in range(pmax - 1)] + ["l1", "l2"]


def _read_family(size_path, data_path, order_prim, pmax):
    sizes = np.fromfile(size_path, dtype=np.int32)
    if sizes.size < 2:
        raise ValueError(f"{size_path}: two ints expected")
    lsize, xsize = int(sizes[0]) - 1, int(sizes[1]) - 1
    if lsize < 1 or xsize < 1:
        raise ValueError(f"{size_path}: sizes {sizes[:2].tolist()}")
    suf = _qtilde_suffixes(order_prim, pmax)
    qt = np.empty((xsize, len(suf), lsize))
    xvec = lvec = None
    for n, sx in enumerate(suf):
        d = array_read(f"{data_path}_{sx}", (lsize + 1) * (xsize + 1)).reshape(lsize + 1, xsize + 1)
        if n == 0:
            xvec, lvec = d[0, 1:].copy(), d[1:, 0].astype(np.int64)
        qt[:, n, :] = d[1:, 1:].T
    return xvec, lvec, qt


def read_qtilde(ini, pmax_prim):
    """read_qtilde (fixed_data.c:2230-2420): the size file holds two native
    ints (lsize + 1, xsize + 1); each data file [lsize + 1][xsize + 1] raw FP64
    has the x grid in row 0, the l values in column 0 and q~_n(l, x_i) at
    [l + 1][i + 1].  Returns {"x", "lvec_T", "qt_T"} with qt_T in the
    [xsize][pmax_prim + 1][lsize] layout of Context.set_transfer, and with
    model:do_polarisation 1 also "lvec_E", "qt_E".  As the reference, rows are
    indexed by position (get_qtilde_T(n, l, x) reads row l)."""
    p = _params(ini)
    names = proj_names(ini)
    x, lT, qT = _read_family(names["T_size"], names["T_data"], p["order_prim"], pmax_prim)
    out = {"x": x, "lvec_T": lT, "qt_T": qT}
    if p["do_polarisation"] == 1:
        xE, lE, qE = _read_family(names["E_size"], names["E_data"], p["order_prim"], pmax_prim)
        if xE.size != x.size:
            raise ValueError(f"E transfer grid has {xE.size} points, T has {x.size}")
        out.update(lvec_E=lE, qt_E=qE)
    return out


def _write_family(size_path, data_path, order_prim, xvec, lvec, qt):
    xsize, P, lsize = qt.shape
    np.array([lsize + 1, xsize + 1], dtype=np.int32).tofile(size_path)
    d = np.zeros((lsize + 1, xsize + 1))
    d[0, 1:] = xvec
    d[1:, 0] = lvec
    for n, sx in enumerate(_qtilde_suffixes(order_prim, P - 1)):
        d[0, 0] = n  # output_qtilde stores the index there; read_qtilde ignores it
        d[1:, 1:] = qt[:, n, :].T
        array_write(f"{data_path}_{sx}", d)


def write_qtilde(ini, xvec, qt_t, qt_e=None, lvec_t=None, lvec_e=None):
    """The files read_qtilde reads (output_qtilde, fixed_data.c:2076-2200, plus
    the _l1/_l2 pair of order_prim 4): qt_t [xsize][pmax_prim + 1][lsize],
    lvec defaulting to 0..lsize-1.  Returns proj_names(ini)."""
    p = _params(ini)
    names = proj_names(ini)
    xvec = np.asarray(xvec, dtype=np.float64)
    qt_t = np.asarray(qt_t, dtype=np.float64)
    lvec_t = np.arange(qt_t.shape[2]) if lvec_t is None else lvec_t
    _write_family(names["T_size"], names["T_data"], p["order_prim"], xvec, lvec_t, qt_t)
    if qt_e is not None:
        qt_e = np.asarray(qt_e, dtype=np.float64)
        lvec_e = np.arange(qt_e.shape[2]) if lvec_e is None else lvec_e
        _write_family(names["E_size"], names["E_data"], p["order_prim"], xvec, lvec_e, qt_e)
    return names


# ------------------------------------------------------------ the drivers

def _late_setup(ini, basis_t, basis_e, pol_orders, spectra, pol=None):
    """The driver's view of set_terms_late + create_basis_late: mode lists from
    the INI file (pol_orders overrides the polarised ones) and the basis tables
    given, or built by basis_late when basis_t is None."""
    p = _params(ini)
    N = p["terms"]
    pol = p["do_polarisation"] == 1 if pol is None else pol
    lo = late_orders(ini, N, pol, pol_orders)
    tri = lo["ttt"]
    if basis_t is None:
        if spectra is None and p["order_late"] in (5, 6):
            spectra = load_spectra(ini, lens=p["order_late"] == 6, tl=p["order_late"] == 5)
        basis_t, be = basis_late(ini, lo["pmax_T"], lo["pmax_E"] if pol else None, spectra, pol)
        basis_e = be if basis_e is None else basis_e
    basis_t = np.asarray(basis_t, dtype=np.float64)
    L = p["T_lmax"] - p["T_lmin"] + 1
    if basis_t.ndim != 2 or basis_t.shape[0] != L:
        raise ValueError(f"basis_T has {basis_t.shape[0]} rows, T_lmin..T_lmax needs {L}")
    if tri.max() >= basis_t.shape[1]:
        raise ValueError(f"mode index {tri.max()} needs more than {basis_t.shape[1]} basis functions")
    if pol:
        if basis_e is None:
            raise ValueError("do_polarisation needs the E basis")
        basis_e = np.asarray(basis_e, dtype=np.float64)
        pol_orders = [np.ascontiguousarray(lo[k]) for k in ("tte", "tee", "eee")]
    return p, N, tri, basis_t, basis_e, pol_orders, pol


def ortho_late(ini_path, basis_t=None, basis_e=None, pol_orders=None, split=False, device=0, spectra=None):
    """ortho_late_mpi.c on the GPU: Gamma of the TTT modes (and TTE/TEE/EEE with
    do_polarisation), the orthogonalisation of each (gflag_pca as old:gflag_pca),
    and orthol_XXX / lambdal_XXX written where output_orthol / output_lambdal
    (fixed_data.c:3453-3469, 3749-3765) put them.  Mode lists from the INI
    (late_orders; pol_orders [TTE, TEE, EEE] with T indices first overrides the
    polarised ones).  basis_t [L_T][P_T] on T_lmin..T_lmax, or None for
    basis_late's tables (spectra for order_late 6).  Returns the dict of
    written paths."""
    import modal_gb300 as mg
    ini = read_ini(ini_path)
    p, N, tri, basis_t, basis_e, pol_orders, pol = _late_setup(ini, basis_t, basis_e, pol_orders, spectra)
    names = output_names(ini)
    written = {}
    with mg.Context(device) as c:
        c.set_basis(p["T_lmin"], p["T_lmax"], basis_t)
        c.set_modes(tri)
        if pol:
            c.set_basis_e(p["E_lmin"], p["E_lmax"], basis_e)
            c.set_modes_pol(*pol_orders)
        c.init_glint()
        G = {"TTT": c.gamma(mg.PREC_SPLIT if split else mg.PREC_FP64)}
        if pol:
            G["TTE"], G["TEE"], G["EEE"] = c.gamma_pol()
        for x, g in G.items():
            o, lam, _, _ = c.orthogonalise(g, pca_flag=p["gflag_pca"])
            for fam, arr in (("orthol", o), ("lambdal", lam)):
                key = f"{fam}_{x}"
                if key in names:
                    array_write(names[key], arr)
                    written[key] = names[key]
    return written


def gamma_late(ini_path, basis_t, cl_total, basis_e=None, pol_orders=None, spec9=None, device=0, spectra=None):
    """gamma_mpi.c on the GPU: the late x primordial Gamma of the INI file's
    modes from the transfer files, turned by orthoinv = lambdal^T lambdal
    (gamma_mpi.c:260-291, 800-840) and written as gamma_XXX (output_gamma,
    fixed_data.c:3077-3091: terms^2 raw FP64, row = late mode).

    basis:do3D 0 takes the 3D path (calculate_gamma_TTT_3D_nested; as the
    reference, polarisation is skipped there with a warning and its gamma
    files are written as zeros), any other value
    the 2D one (calculate_gamma_2d, with TTE/TEE/EEE when
    model:do_polarisation is 1).  The lambdal_XXX files are the ones
    ortho_late wrote for the same INI.  Mode lists and basis tables as for
    ortho_late (basis_t None: basis_late's); cl_total over l = 0..T_lmax
    (C_l + N_l/b_l^2); with polarisation spec9 [9][T_lmax + 1]; either None:
    load_spectra's, from the INI's spectrum files.  Returns the dict of
    written paths."""
    import warnings

    import modal_gb300 as mg
    ini = read_ini(ini_path)
    p0 = _params(ini)
    lmax = p0["T_lmax"]
    do3d = getint(ini, "basis:do3D", 1) == 0
    pol = p0["do_polarisation"] == 1
    if pol and do3d:
        warnings.warn("polarisation currently disabled for 3D gamma calculations: skipping it")
    if cl_total is None or (pol and not do3d and spec9 is None):
        sp = load_spectra(ini)
        cl_total = sp["cl_total"] if cl_total is None else cl_total
        spec9 = sp.get("spec9") if spec9 is None else spec9
    cl_total = np.asarray(cl_total, dtype=np.float64).ravel()
    if cl_total.size < lmax + 1:
        raise ValueError(f"cl_total has {cl_total.size} values, l = 0..{lmax} needs {lmax + 1}")
    p, N, tri, basis_t, basis_e, pol_orders, pol = _late_setup(ini, basis_t, basis_e, pol_orders, spectra,
                                                               pol and not do3d)
    prim, pmax = prim_order(ini, N)
    qt = read_qtilde(ini, pmax)
    if qt["qt_T"].shape[2] < lmax + 1:  # the reference reads rows 0..T_lmax
        raise ValueError(f"transfer files hold {qt['qt_T'].shape[2]} l rows, T_lmax = {lmax} needs {lmax + 1}")
    dphi = getdouble(ini, "model:delta_phi", 1.5714e-8)
    names = output_names(ini)
    G = {}
    with mg.Context(device) as c:
        c.set_basis(p["T_lmin"], lmax, basis_t)
        c.set_modes(tri)
        c.set_spectrum(cl_total)
        c.set_transfer(qt["x"], np.ascontiguousarray(qt["qt_T"][:, :, :lmax + 1]), prim)
        if do3d:
            G["TTT"] = c.gamma_transfer_3d(dphi)
        else:
            G["TTT"] = c.gamma_transfer(dphi)
            if pol:
                if spec9 is None:
                    raise ValueError("do_polarisation needs the spectra (spec9)")
                if qt["qt_T"].shape[2] != qt["qt_E"].shape[2]:
                    raise ValueError("the T and E transfer files must hold the same l rows")
                c.set_basis_e(p["E_lmin"], p["E_lmax"], basis_e)
                c.set_modes_pol(*pol_orders)
                spec = np.asarray(spec9, dtype=np.float64).reshape(9, -1)[:, :lmax + 1]
                c.set_transfer_pol(np.ascontiguousarray(qt["qt_E"][:, :, :lmax + 1]), list(spec),
                                   getdouble(ini, "model:fskyT", 1.0), getdouble(ini, "model:fskyE", 1.0))
                G["TTE"], G["TEE"], G["EEE"] = c.gamma_transfer_pol(dphi)
    written = {}
    for x, g in G.items():
        lam = array_read(names[f"lambdal_{x}"], N * N).reshape(N, N)
        array_write(names[f"gamma_{x}"], (lam.T @ lam) @ g)
        written[f"gamma_{x}"] = names[f"gamma_{x}"]
    if do3d and p0["do_polarisation"] == 1:
        # the 3D path leaves the polarised Gammas at zero and output_gamma still
        # writes them (gamma_mpi.c:335-355, fixed_data.c:3085-3089)
        for x in ("TTE", "TEE", "EEE"):
            if f"gamma_{x}" in names:
                array_write(names[f"gamma_{x}"], np.zeros((N, N)))
                written[f"gamma_{x}"] = names[f"gamma_{x}"]
    return written


def modes_suffix(ini, model, p1=0, p2=0, p3=0):
    """output_modes' file suffix (fixed_data.c:3953-3995): _<model>, then
    _<p1>_<p2>_<p3> down to the last shape parameter whose model:shapeX_end is
    non-zero (each p taken when its own _end is non-zero, else 0)."""
    ends = [getint(ini, f"model:shape{k}_end", 0) for k in (1, 2, 3)]
    ps = [p1, p2, p3]
    last = max((k for k in range(3) if ends[k] != 0), default=-1)
    return f"_{model}" + "".join(f"_{ps[k] if ends[k] != 0 else 0}" for k in range(last + 1))


def modes_late(ini_path, basis_t, cl_total, shapes, models, prec=None, device=0, spectra=None):
    """eigenmodetoday_mpi.c on the GPU for shapes given as separable tables or
    bumps (the shape descriptors of Context.project): beta of each shape over
    the tetrapyd, alpha = lambdal^T lambdal beta with orthol/lambdal read from
    the files ortho_late wrote (read_orthol / read_lambdal), written as
    modes_TTT + modes_suffix(model) (output_modes: N raw FP64), and modesR from
    the lower triangle of orthol (eigenmodetoday_mpi.c:148-162, 286-316; the
    reference keeps modesR in memory).  models: the model number of each shape
    (the reference's mode argument; 999 and 998 name its ISW and point-source
    templates, which are not restated).  cl_total None: load_spectra's.
    Returns (written paths, alpha [S][N], modesR [S][N])."""
    import modal_gb300 as mg
    ini = read_ini(ini_path)
    if len(models) != len(shapes):
        raise ValueError(f"{len(shapes)} shapes but {len(models)} model numbers")
    p, N, tri, basis_t, _, _, _ = _late_setup(ini, basis_t, None, None, spectra, pol=False)
    lmax = p["T_lmax"]
    if cl_total is None:
        cl_total = load_spectra(ini)["cl_total"]
    cl_total = np.asarray(cl_total, dtype=np.float64).ravel()
    if cl_total.size < lmax + 1:
        raise ValueError(f"cl_total has {cl_total.size} values, l = 0..{lmax} needs {lmax + 1}")
    names = output_names(ini)
    orthol = array_read(names["orthol_TTT"], N * N).reshape(N, N)
    lambdal = array_read(names["lambdal_TTT"], N * N).reshape(N, N)
    with mg.Context(device) as c:
        c.set_basis(p["T_lmin"], lmax, basis_t)
        c.set_modes(tri)
        c.set_spectrum(cl_total[:lmax + 1])
        c.set_ortho(orthol, lambdal)
        beta = c.project(shapes, mg.PREC_FP64 if prec is None else prec)
        alpha, modes_r = c.alpha(len(shapes), beta)
    written = {}
    for s, m in enumerate(models):
        path = names["modes_TTT"] + modes_suffix(ini, m)
        array_write(path, alpha[s])
        written[f"modes_TTT_{m}"] = path
    return written, alpha, modes_r


def load_txt_int(path, columns=1):
    """load_txt_int (io.c:28-60): '#' lines skipped, the first `columns`
    numbers of every other line as (int)strtod (a blank line reads as zeros).
    A missing file gives an empty list (the reference reports the error and
    reads nothing)."""
    if not os.path.exists(path):
        return np.zeros((0, columns), dtype=np.int32)
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                continue
            toks = line.split()[:columns]
            rows.append([int(_atof(t)) for t in toks] + [0] * (columns - len(toks)))
    return np.array(rows, dtype=np.int32).reshape(-1, columns)


def prune_late(ini_path, gamma_path=None, faillist_path=None, out=None, device=0):
    """basis_optimisation_mpi.c on the GPU: greedy elimination of the late
    modes that keeps the smallest eigenvalue of the normalised Gamma largest.
    Gamma is read raw [N][N] from gamma_path (the reference reads a
    master_orthol_TTT_<T_lmax>_<E_lmax>_<order_late>_<terms>.unf file under a
    site path; its name under model:directory is the default here) and the
    modes listed in faillist_path (default faillist_TTT_<T_lmax>_<order_late>_
    <terms>.txt there; absent: none) are left out.  Prints the reference's lines
    (basis_optimisation_mpi.c:141-176, 326-343): the left-out and active modes,
    then per elimination "index i j k lambda_min time" and the survivor with
    1 and 0.  Returns (order, lambda_min)."""
    import time

    import modal_gb300 as mg
    out = sys.stdout if out is None else out
    ini = read_ini(ini_path)
    p = _params(ini)
    N = p["terms"]
    tri = mode_order(ini, N)
    d = p["directory"]
    tag = f"{p['T_lmax']}_{p['order_late']}_{N}"
    gamma_path = gamma_path or f"{d}master_orthol_TTT_{p['T_lmax']}_{p['E_lmax']}_{p['order_late']}_{N}.unf"
    faillist_path = faillist_path or f"{d}faillist_TTT_{tag}.txt"
    G = array_read(gamma_path, N * N).reshape(N, N)
    fail = load_txt_int(faillist_path)[:, 0][:N]
    active = [n for n in range(N) if n not in set(fail.tolist())]
    print(f"terms: {N}", file=out)
    print(f"modes complete\t{fail.size}", file=out)
    for n in fail.tolist():
        print("%d\t%d\t%d\t%d" % (n, *tri[n]), file=out)
    print(f"modes active\t{len(active)}", file=out)
    for n in active:
        print("%d\t%d\t%d\t%d" % (n, *tri[n]), file=out)
    print("starting reduction", file=out)
    t0 = time.perf_counter()
    with mg.Context(device) as c:
        order, lam = c.basis_prune(G, fail)
    dt = (time.perf_counter() - t0) / max(1, order.size - 1)
    for r in range(order.size - 1):
        n = int(order[r])
        print("%d\t%d\t%d\t%d\t%e\t%e" % (n, *tri[n], lam[r], dt), file=out)
    if order.size:
        n = int(order[-1])
        print("%d\t%d\t%d\t%d\t%e\t%e" % (n, *tri[n], 1.0, 0.0), file=out)
    return order, lam


BASIS_HELP = "raw FP64 [L_T][P_T] (needs --pt); omitted: create_basis_late's table for basis:order_late"
CL_HELP = "raw FP64 C_l + N_l/b_l^2 over l = 0..T_lmax; omitted: from the INI's cls/BN/pixel-window files"


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    o = sub.add_parser("ortho_late", help="Gamma + orthogonalisation with the reference's file names")
    o.add_argument("ini")
    o.add_argument("basis_t", nargs="?", help=BASIS_HELP)
    o.add_argument("--pt", type=int, help="P_T, the number of T basis functions")
    o.add_argument("--basis-e", help="raw FP64 [L_E][P_E]")
    o.add_argument("--pe", type=int, help="P_E")
    o.add_argument("--split", action="store_true", help="split-precision Gamma")
    g = sub.add_parser("gamma_late", help="late x primordial Gamma from the transfer files, gamma_XXX written")
    g.add_argument("ini")
    g.add_argument("basis_t", nargs="?", help=BASIS_HELP)
    g.add_argument("--pt", type=int, help="P_T, the number of T basis functions")
    g.add_argument("--cl", help=CL_HELP)
    g.add_argument("--basis-e", help="raw FP64 [L_E][P_E]")
    g.add_argument("--pe", type=int, help="P_E")
    g.add_argument("--spec9", help="raw FP64 [9][T_lmax+1] spectra, beams and noise")
    pr = sub.add_parser("prune_late", help="greedy mode elimination (basis_optimisation_mpi), printed")
    pr.add_argument("ini")
    pr.add_argument("--gamma", help="raw FP64 [N][N] Gamma (default: master_orthol_TTT_... under model:directory)")
    pr.add_argument("--faillist", help="modes to leave out, one per line (default: faillist_TTT_... there)")
    m = sub.add_parser("modes_late", help="modes of a separable shape with the orthol/lambdal files, modes_TTT written")
    m.add_argument("ini")
    m.add_argument("basis_t", nargs="?", help=BASIS_HELP)
    m.add_argument("--pt", type=int, help="P_T, the number of T basis functions")
    m.add_argument("--cl", help=CL_HELP)
    m.add_argument("--tab", required=True, help=".npy separable shape table [T][3][T_lmax+1]")
    m.add_argument("--model", type=int, required=True, help="model number in the output name")
    a = ap.parse_args(argv)
    if a.cmd == "prune_late":
        prune_late(a.ini, a.gamma, a.faillist)
        return
    if a.basis_t is not None and a.pt is None:
        ap.error("a basis file needs --pt")
    bt = array_read(a.basis_t).reshape(-1, a.pt) if a.basis_t is not None else None
    if a.cmd == "modes_late":
        import modal_gb300 as mg
        shape = {"kind": mg.SHAPE_SEPARABLE, "tab": np.load(a.tab)}
        out, _, _ = modes_late(a.ini, bt, array_read(a.cl) if a.cl else None, [shape], [a.model])
        for k, v in out.items():
            print(k, v)
        return
    be = array_read(a.basis_e).reshape(-1, a.pe) if a.basis_e else None
    if a.cmd == "ortho_late":
        out = ortho_late(a.ini, bt, be, None, a.split)
    else:
        sp = array_read(a.spec9).reshape(9, -1) if a.spec9 else None
        out = gamma_late(a.ini, bt, array_read(a.cl) if a.cl else None, be, None, sp)
    for k, v in out.items():
        print(k, v)


if __name__ == "__main__":
    main()
