"""Reference-compatible file formats and an INI-driven driver for the GPU path.

The reference's drivers read an iniparser INI file (parameter.c:127-980), name
their outputs from its keys (parameter.c:243-700), and write raw native FP64
arrays (array_write / array_read, arrays.c:6-77).  This module restates those
conventions so that results of the GPU path land in the files the reference's
later stages read:

  read_ini(path)                     -> {"section:key": "value"} (iniparser keys)
  output_names(ini)                  -> the orthol/lambdal/modes/gamma file names
  array_write(path, a) / array_read  -> raw native FP64, no header
  load_three_int(path)               -> [n][3] mode orderings (io.c:229-257)
  mode_order(ini, N)                 -> set_terms_late orderings 1, 2 and 3
  ortho_late(ini_path, basis_t, ...) -> ortho_late_mpi.c's outputs from the GPU

Command line:
  python modal_files.py ortho_late <ini> <basis_T.unf> [--basis-e <basis_E.unf>]
      [--pol-orders TTE TEE EEE] [--split]
basis files are raw FP64 [L][P] tables (basis_late_T / basis_late_E layouts,
fixed_data.c:1764), as the reference's create_basis_late would fill them.
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
    with surrounding quotes removed; ';' and '#' start comments."""
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
            if val[:1] in "\"'":
                q = val[0]
                end = val.find(q, 1)
                val = val[1:end] if end > 0 else val[1:]
            else:
                val = re.split(r"\s[;#]", val, maxsplit=1)[0].strip()
            out[f"{section}:{key.strip().lower()}"] = val
    return out


def _get(ini, key, default, conv=str):
    v = ini.get(key.lower())
    if v is None:
        return default
    try:
        return conv(v)
    except ValueError:
        return default


def getint(ini, key, default):
    return _get(ini, key, default, lambda v: int(float(v)) if v.strip() else default)


def getdouble(ini, key, default):
    return _get(ini, key, default, float)


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


def mode_order(ini, N):
    """TTT mode triples of set_terms_late for basis:order_late 1, 2 or 3
    (3: read from model:order_TTT_file_late)."""
    case = getint(ini, "basis:order_late", 3)
    if case == 1:
        return _order_case1(N)
    if case == 2:
        return _order_case2(N)
    p = _params(ini)
    f = getstring(ini, "model:order_TTT_file_late", "order_dist.txt")
    path = f if f.startswith("/") else p["directory"] + f
    t = load_three_int(path)
    if t.shape[0] < N:
        raise ValueError(f"eigenfunction {N} exceeds that in TTT distance file {path}")
    return t[:N]


# ------------------------------------------------------------ the driver

def ortho_late(ini_path, basis_t, basis_e=None, pol_orders=None, split=False, device=0):
    """ortho_late_mpi.c on the GPU: Gamma of the TTT modes (and TTE/TEE/EEE with
    do_polarisation), the orthogonalisation of each (gflag_pca as old:gflag_pca),
    and orthol_XXX / lambdal_XXX written where output_orthol / output_lambdal
    (fixed_data.c:3453-3469, 3749-3765) put them.  basis_t [L_T][P_T] on
    T_lmin..T_lmax.  Returns the dict of written paths."""
    import modal_gb300 as mg
    ini = read_ini(ini_path)
    p = _params(ini)
    N = p["terms"]
    basis_t = np.asarray(basis_t, dtype=np.float64)
    L = p["T_lmax"] - p["T_lmin"] + 1
    if basis_t.shape[0] != L:
        raise ValueError(f"basis_T has {basis_t.shape[0]} rows, T_lmin..T_lmax needs {L}")
    tri = mode_order(ini, N)
    if tri.max() >= basis_t.shape[1]:
        raise ValueError(f"mode index {tri.max()} needs more than {basis_t.shape[1]} basis functions")
    names = output_names(ini)
    written = {}
    with mg.Context(device) as c:
        c.set_basis(p["T_lmin"], p["T_lmax"], basis_t)
        c.set_modes(tri)
        pol = p["do_polarisation"] == 1
        if pol:
            if basis_e is None or pol_orders is None:
                raise ValueError("do_polarisation needs the E basis and the TTE/TEE/EEE orders")
            c.set_basis_e(p["E_lmin"], p["E_lmax"], np.asarray(basis_e, dtype=np.float64))
            c.set_modes_pol(*[np.asarray(o, dtype=np.int32)[:N] for o in pol_orders])
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


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    o = sub.add_parser("ortho_late", help="Gamma + orthogonalisation with the reference's file names")
    o.add_argument("ini")
    o.add_argument("basis_t", help="raw FP64 [L_T][P_T]")
    o.add_argument("--pt", type=int, required=True, help="P_T, the number of T basis functions")
    o.add_argument("--basis-e", help="raw FP64 [L_E][P_E]")
    o.add_argument("--pe", type=int, help="P_E")
    o.add_argument("--pol-orders", nargs=3, metavar=("TTE", "TEE", "EEE"))
    o.add_argument("--split", action="store_true", help="split-precision Gamma")
    a = ap.parse_args(argv)
    bt = array_read(a.basis_t).reshape(-1, a.pt)
    be = array_read(a.basis_e).reshape(-1, a.pe) if a.basis_e else None
    po = [load_three_int(f) for f in a.pol_orders] if a.pol_orders else None
    for k, v in ortho_late(a.ini, bt, be, po, a.split).items():
        print(k, v)


if __name__ == "__main__":
    main()
