"""CPU oracle for the Modal-CMB mode-space hot path -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker or the timed CPU baseline; the product
(libmodal_gb300.so) never calls it.

Two CPU implementations are exposed:
  * Oracle: the plain-C restatement in oracle/modal_oracle.c (builds anywhere);
  * Ref:    the reference's own sources compiled in place with stand-in
            headers (oracle/_ref/libmodalref.so, built by `make -C oracle ref`
            when the reference checkout is present).
The PCA branch of the orthogonalisation (gsl_eigen_symmv, absent here) is
restated with numpy.linalg.eigh, following ortho_late_mpi.c:775-805.
"""
import contextlib
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libmodaloracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmodalref.so")
# the reference checkout (only for compiling it in place; absent on GPU machines)
REFERENCE_DIR = os.environ.get("MODAL_REFERENCE_DIR", "/root/reference")


def _shape_args(shape):
    """(kind, nterms, tab, centre, sigma) of a shape dict for the C drivers."""
    if shape["kind"] == 0:
        tab = np.ascontiguousarray(shape["tab"], dtype=np.float64)
        return 0, tab.shape[0], tab, (0.0, 0.0, 0.0), 1.0
    c = shape["c"]
    return 1, 0, None, (float(c[0]), float(c[1]), float(c[2])), float(shape["sigma"])


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


def build_ref():
    """Compile the reference's hot-path sources in place (needs the checkout)."""
    if not os.path.isdir(REFERENCE_DIR):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REFERENCE_DIR], check=True)
    return REF_SO


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@contextlib.contextmanager
def quiet_stdout():
    """Silence C-level printf (the reference prints progress lines)."""
    import sys
    sys.stdout.flush()
    fd = os.dup(1)
    null = os.open(os.devnull, os.O_WRONLY)
    os.dup2(null, 1)
    try:
        yield
    finally:
        ctypes.CDLL(None).fflush(None)
        os.dup2(fd, 1)
        os.close(fd)
        os.close(null)


class Oracle:
    """ctypes view of oracle/modal_oracle.c."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        L = ctypes.CDLL(path)
        vp, i, l, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double
        for name, res, args in [
            ("orc_gl_nodes", i, [i, vp, vp]),
            ("orc_legendre_table", i, [i, i, vp, vp]),
            ("orc_basis_legendre", i, [i, i, d, d, vp, vp]),
            ("orc_mij", i, [i, i, i, i, vp, vp, vp]),
            ("orc_orthol_pair", i, [i, i, vp, vp, vp, i, i, vp]),
            ("orc_gamma", i, [i, vp, i, i, vp, vp, i, vp]),
            ("orc_gamma_sample", l, [i, vp, i, i, vp, vp, i, l, vp]),
            ("orc_geometric", d, [i, i, i]),
            ("orc_permsix", d, [i, i, i]),
            ("orc_tetrapyd_next", i, [i, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]),
            ("orc_tetrapyd_count", l, [i, i]),
            ("orc_plijk", d, [vp, i, vp, i, i, i, i, i, i]),
            ("orc_project", i, [i, i, i, vp, i, vp, vp, i, i, vp, d, d, d, d, i, l, vp]),
            ("orc_ortho_cholesky", l, [i, vp, vp, vp]),
            ("orc_alpha", i, [i, vp, vp, vp, vp, vp]),
            ("orc_modify_bispectrum", i, [i, vp, vp, vp, vp, vp]),
            ("orc_calculate_modes", i, [i, i, i, vp, i, vp, i, vp, vp]),
            ("orc_integrate_cubic_spline", d, [vp, vp, i]),
            ("orc_gamma_transfer", i, [i, i, i, vp, i, vp, vp, i, vp, vp, i, vp, i, vp, i, vp, d, vp]),
            ("orc_gamma_3d", i, [i, i, i, vp, i, vp, vp, i, vp, i, vp, i, vp, d, vp]),
            ("orc_gamma_pol", i, [i, vp, vp, vp, i, i, i, vp, vp, vp, vp, vp, vp]),
            ("orc_gamma_transfer_pol", i, [i, i, i, vp, i, i, i, vp, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                           vp, vp, d, d, i, vp, vp, i, vp, i, vp, vp, i, vp, d, vp]),
            ("orc_prim_weight", d, [i, i, i, i, i]),
            ("orc_prim_walk", l, [i, i, l, vp]),
            ("orc_prim_ortho", i, [i, i, d, i, vp, i, vp, vp]),
            ("orc_prim_eigen", i, [i, i, d, i, vp, i, vp, i, i, vp, d, d, d, d, vp, vp]),
        ]:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        self.L = L

    def gl_nodes(self, n):
        x, w = np.empty(n), np.empty(n)
        self.L.orc_gl_nodes(n, _p(x), _p(w))
        return x, w

    def legendre_table(self, mu, lmax):
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        out = np.empty((mu.size, lmax + 1))
        self.L.orc_legendre_table(mu.size, lmax, _p(mu), _p(out))
        return out

    def basis_legendre(self, values, pmax, vmin, vmax):
        values = np.ascontiguousarray(values, dtype=np.float64)
        out = np.empty((values.size, pmax + 1))
        self.L.orc_basis_legendre(values.size, pmax, float(vmin), float(vmax), _p(values), _p(out))
        return out

    def mij(self, gl_pl, lmin, lmax, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        gl_pl = np.ascontiguousarray(gl_pl, dtype=np.float64)
        P = q.shape[1]
        out = np.empty((P, P, gl_pl.shape[0]))
        self.L.orc_mij(gl_pl.shape[0], lmin, lmax, P, _p(gl_pl), _p(q), _p(out))
        return out

    def gamma(self, M, w, triples, nthreads=0):
        triples = np.ascontiguousarray(triples, dtype=np.int32)
        M = np.ascontiguousarray(M)
        w = np.ascontiguousarray(w, dtype=np.float64)
        N = triples.shape[0]
        out = np.empty((N, N))
        self.L.orc_gamma(N, _p(triples), M.shape[0], M.shape[2], _p(M), _p(w), nthreads, _p(out))
        return out

    def gamma_sample(self, M, w, triples, npairs, nthreads=0):
        triples = np.ascontiguousarray(triples, dtype=np.int32)
        out = np.empty(max(1, npairs))
        n = self.L.orc_gamma_sample(triples.shape[0], _p(triples), M.shape[0], M.shape[2], _p(M), _p(w),
                                    nthreads, npairs, _p(out))
        return out[:n]

    def orthol_pair(self, M, w, triples, m, n):
        triples = np.ascontiguousarray(triples, dtype=np.int32)
        r = np.zeros(4)
        self.L.orc_orthol_pair(M.shape[0], M.shape[2], _p(M), _p(w), _p(triples), m, n, _p(r))
        return r[0]

    def geometric(self, i, j, k):
        return self.L.orc_geometric(i, j, k)

    def tetrapyd_count(self, lmin, lmax):
        return self.L.orc_tetrapyd_count(lmin, lmax)

    def project(self, lmin, lmax, q, triples, cl, shape, nthreads=0, max_points=0):
        q = np.ascontiguousarray(q, dtype=np.float64)
        triples = np.ascontiguousarray(triples, dtype=np.int32)
        cl = np.ascontiguousarray(cl, dtype=np.float64)
        N = triples.shape[0]
        beta = np.empty(N)
        if shape["kind"] == 0:
            tab = np.ascontiguousarray(shape["tab"], dtype=np.float64)
            args = (0, tab.shape[0], _p(tab), 0.0, 0.0, 0.0, 1.0)
        else:
            tab = None
            c = shape["c"]
            args = (1, 0, None, float(c[0]), float(c[1]), float(c[2]), float(shape["sigma"]))
        self.L.orc_project(lmin, lmax, q.shape[1], _p(q), N, _p(triples), _p(cl), *args, nthreads, max_points,
                           _p(beta))
        return beta

    def modify_bispectrum(self, b, vec, cl, beam=None, noise=None):
        b = np.array(b, dtype=np.float64, order="C", copy=True)
        size = b.shape[0]
        vec = np.ascontiguousarray(vec, dtype=np.int32)
        beam = np.ones(size) if beam is None else np.ascontiguousarray(beam, dtype=np.float64)
        noise = np.zeros(size) if noise is None else np.ascontiguousarray(noise, dtype=np.float64)
        cl = np.ascontiguousarray(cl[:size], dtype=np.float64)
        self.L.orc_modify_bispectrum(size, _p(vec), _p(cl), _p(beam), _p(noise), _p(b))
        return b

    def calculate_modes(self, lmin, lmax, q, triples, b):
        q = np.ascontiguousarray(q, dtype=np.float64)
        triples = np.ascontiguousarray(triples, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.float64)
        beta = np.empty(triples.shape[0])
        self.L.orc_calculate_modes(lmin, lmax, q.shape[1], _p(q), triples.shape[0], _p(triples), b.shape[0], _p(b),
                                   _p(beta))
        return beta

    def integrate_cubic_spline(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        return self.L.orc_integrate_cubic_spline(_p(x), _p(y), x.size)

    def gamma_transfer(self, lmin, lmax, q, triples, cl, mu, w, xvec, qt, prim, dphi):
        q = np.ascontiguousarray(q, dtype=np.float64)
        triples = np.ascontiguousarray(triples, dtype=np.int32)
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        qt = np.ascontiguousarray(qt, dtype=np.float64)
        xvec = np.ascontiguousarray(xvec, dtype=np.float64)
        N, Nprim = triples.shape[0], prim.shape[0]
        out = np.empty((N, Nprim))
        self.L.orc_gamma_transfer(lmin, lmax, q.shape[1], _p(q), N, _p(triples), _p(np.ascontiguousarray(cl)), mu.size,
                                  _p(np.ascontiguousarray(mu)), _p(np.ascontiguousarray(w)), xvec.size, _p(xvec),
                                  qt.shape[1], _p(qt), Nprim, _p(prim), float(dphi), _p(out))
        return out

    def gamma_3d(self, lmin, lmax, q, triples, cl, xvec, qt, prim, dphi):
        """[N][Nprim]: calculate_gamma_TTT_3D_nested's 3D transfer Gamma (any N, Nprim)."""
        q, cl, xvec, qt = (np.ascontiguousarray(a, dtype=np.float64) for a in (q, cl, xvec, qt))
        triples, prim = (np.ascontiguousarray(a, dtype=np.int32) for a in (triples, prim))
        N, Nprim = triples.shape[0], prim.shape[0]
        out = np.empty((N, Nprim))
        self.L.orc_gamma_3d(lmin, lmax, q.shape[1], _p(q), N, _p(triples), _p(cl), xvec.size, _p(xvec), qt.shape[1],
                            _p(qt), Nprim, _p(prim), float(dphi), _p(out))
        return out

    def gamma_pol(self, MT, ME, w, tte, tee, eee):
        """(Gamma_TTE, Gamma_TEE, Gamma_EEE) from Mij_T / Mij_E [P][P][nmu]."""
        MT, ME = np.ascontiguousarray(MT), np.ascontiguousarray(ME)
        w = np.ascontiguousarray(w, dtype=np.float64)
        t = [np.ascontiguousarray(x, dtype=np.int32) for x in (tte, tee, eee)]
        N = t[0].shape[0]
        outs = [np.empty((N, N)) for _ in range(3)]
        self.L.orc_gamma_pol(N, _p(t[0]), _p(t[1]), _p(t[2]), MT.shape[0], ME.shape[0], MT.shape[2], _p(MT), _p(ME),
                             _p(w), _p(outs[0]), _p(outs[1]), _p(outs[2]))
        return tuple(outs)

    def gamma_transfer_pol(self, lmin, lmax, qT, lminE, lmaxE, qE, tte, tee, eee, spec9, fsky_t, fsky_e, mu, w,
                           xvec, qtT, qtE, prim, dphi):
        """[3][N][Nprim]: TTE, TEE, EEE transfer Gamma (spec9 = cl_tt, cl_te, cl_ee, b_tt, b_te, b_ee,
        n_tt, n_te, n_ee over l = 0..lmax)."""
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        ii = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
        qT, qE, spec9, mu, w, xvec, qtT, qtE = map(f, (qT, qE, spec9, mu, w, xvec, qtT, qtE))
        tte, tee, eee, prim = map(ii, (tte, tee, eee, prim))
        N, Nprim = tte.shape[0], prim.shape[0]
        out = np.empty((3, N, Nprim))
        sp = [spec9[i] for i in range(9)]
        sp = [np.ascontiguousarray(x) for x in sp]
        self.L.orc_gamma_transfer_pol(lmin, lmax, qT.shape[1], _p(qT), lminE, lmaxE, qE.shape[1], _p(qE), N, _p(tte),
                                      _p(tee), _p(eee), *[_p(x) for x in sp], float(fsky_t), float(fsky_e), mu.size,
                                      _p(mu), _p(w), xvec.size, _p(xvec), qtT.shape[1], _p(qtT), _p(qtE), Nprim,
                                      _p(prim), float(dphi), _p(out))
        return out

    def prim_walk(self, kmin, kmax_i):
        n = self.L.orc_prim_walk(kmin, kmax_i, 0, None)
        pts = np.empty((n, 3), dtype=np.int32)
        self.L.orc_prim_walk(kmin, kmax_i, n, _p(pts))
        return pts

    def prim_ortho(self, kmin, kmax_i, kmax, basis, prim):
        """calculate_ortho: packed upper triangle [N(N+1)/2] of the k-grid Gram matrix."""
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        N = prim.shape[0]
        out = np.empty(N * (N + 1) // 2)
        self.L.orc_prim_ortho(kmin, kmax_i, float(kmax), basis.shape[1], _p(basis), N, _p(prim), _p(out))
        return out

    def prim_eigen(self, kmin, kmax_i, kmax, basis, prim, shape):
        """calculate_eigen + integrate_template2 for one shape: (alpha[N], <S,S>)."""
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        N = prim.shape[0]
        a, n2 = np.empty(N), np.empty(1)
        kind, nterms, tab, c, sigma = _shape_args(shape)
        self.L.orc_prim_eigen(kmin, kmax_i, float(kmax), basis.shape[1], _p(basis), N, _p(prim), kind, nterms,
                              _p(tab), c[0], c[1], c[2], sigma, _p(a), _p(n2))
        return a, n2[0]

    def ortho_cholesky(self, gamma):
        """Cholesky branch; returns (orthol, lambdal, fail) with fail = -1 or the failing pivot row."""
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        N = g.shape[0]
        o, lam = np.empty((N, N)), np.empty((N, N))
        r = self.L.orc_ortho_cholesky(N, _p(g), _p(o), _p(lam))
        return o, lam, (r - 1 if r > 0 else -1)

    def alpha(self, orthol, lambdal, beta):
        N = orthol.shape[0]
        a, m = np.empty(N), np.empty(N)
        self.L.orc_alpha(N, _p(np.ascontiguousarray(orthol)), _p(np.ascontiguousarray(lambdal)),
                         _p(np.ascontiguousarray(beta, dtype=np.float64)), _p(a), _p(m))
        return a, m


def ortho_pca(gamma, floor=0.0):
    """PCA branch of ortho_late_mpi.c:775-805 with numpy.linalg.eigh standing
    in for gsl_eigen_symmv (eigenvalues sorted descending).  floor > 0 keeps
    only eigenvalues above floor * e_max (the reference's rule is floor 0).
    Returns (lambdainv, lambda, r)."""
    norm = np.sqrt(np.diag(gamma))
    gh = gamma / np.outer(norm, norm)
    e, V = np.linalg.eigh(gh)
    e, V = e[::-1], V[:, ::-1]
    cut = floor * e[0] if floor > 0.0 else 0.0
    r = 0
    for i in range(len(e)):
        if e[i] > cut:
            r = i + 1
        else:
            break
    N = len(e)
    lam = np.zeros((N, N))
    inv = np.zeros((N, N))
    lam[:r] = V[:, :r].T / (norm[None, :] * np.sqrt(e[:r])[:, None])
    inv[:, :r] = norm[:, None] * V[:, :r] * np.sqrt(e[:r])[None, :]
    return inv, lam, r


class Ref:
    """ctypes view of the reference compiled in place (oracle/_ref)."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            if build_ref() is None:
                raise FileNotFoundError("reference checkout not present; oracle/_ref cannot be built")
        L = ctypes.CDLL(path)
        vp, i, l, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double
        for name, res, args in [
            ("ref_setup", i, [i, i, i, vp, i, vp, vp]),
            ("ref_asy", i, [i, vp, vp]),
            ("ref_legendre_Pl", d, [i, d]),
            ("ref_basis_legendre", i, [i, i, d, d, vp, vp]),
            ("ref_basis_family", i, [i, i, i, d, d, vp, vp]),
            ("ref_init_gamma", i, []),
            ("ref_orthol_pair", i, [i, i, vp]),
            ("ref_gamma", l, [i, l, vp]),
            ("ref_geometric", d, [i, i, i]),
            ("ref_plijk", d, [i, i, i, i]),
            ("ref_tetrapyd_walk", l, [i, i, l, vp]),
            ("ref_decompose", i, [i, i, i, vp]),
            ("ref_project", i, [i, i, i, vp, d, d, d, d, l, vp]),
            ("ref_modify_bispectrum", i, [i, vp, vp]),
            ("ref_calculate_modes", i, [i, vp, vp]),
            ("ref_gamma_transfer", i, [i, vp, i, vp, i, vp, d, vp]),
            ("ref_gamma_3d", i, [i, vp, i, vp, i, vp, d, vp]),
            ("ref_setup_pol", i, [i, i, i, vp, vp, vp, vp]),
            ("ref_gamma_pol", i, [vp]),
            ("ref_setup_pol_spectra", i, [i, vp, d, d]),
            ("ref_gamma_transfer_pol", i, [i, vp, i, vp, vp, i, vp, d, vp]),
            ("ref_prim_ortho", i, [i, i, d, i, vp, i, vp, vp]),
            ("ref_prim_eigen", i, [i, i, d, i, vp, i, vp, i, i, vp, d, d, d, d, vp, vp]),
        ]:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        self.L = L
        self._keep = None

    def setup(self, lmin, lmax, q, triples, cl):
        q = np.ascontiguousarray(q, dtype=np.float64)
        triples = np.ascontiguousarray(triples, dtype=np.int32)
        cl = np.ascontiguousarray(cl, dtype=np.float64)
        self.L.ref_setup(lmin, lmax, q.shape[1], _p(q), triples.shape[0], _p(triples), _p(cl))
        self.N = triples.shape[0]

    def asy(self, n):
        x, w = np.empty(n), np.empty(n)
        self.L.ref_asy(n, _p(x), _p(w))
        return x, w

    def basis_legendre(self, values, pmax, vmin, vmax):
        values = np.ascontiguousarray(values, dtype=np.float64)
        out = np.empty((values.size, pmax + 1))
        self.L.ref_basis_legendre(values.size, pmax, float(vmin), float(vmax), _p(values), _p(out))
        return out

    def basis_family(self, kind, values, pmax, vmin, vmax):
        """basis_functions_{legendre, fourier, sinlog, bi} for kind 0..3."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        out = np.empty((values.size, pmax + 1))
        if self.L.ref_basis_family(kind, values.size, pmax, float(vmin), float(vmax), _p(values), _p(out)) != 0:
            raise ValueError(f"basis family {kind} with pmax {pmax}")
        return out

    def init_gamma(self):
        self.L.ref_init_gamma()

    def setup_pol(self, lminE, lmaxE, qE, tte, tee, eee):
        """After setup(): E basis [L_E][P_E] and TTE/TEE/EEE triples (find_perm conventions)."""
        qE = np.ascontiguousarray(qE, dtype=np.float64)
        t = [np.ascontiguousarray(x, dtype=np.int32) for x in (tte, tee, eee)]
        self._keep_pol = (qE, t)
        self.L.ref_setup_pol(lminE, lmaxE, qE.shape[1], _p(qE), _p(t[0]), _p(t[1]), _p(t[2]))

    def gamma_3d(self, xvec, qt, prim, dphi):
        """[N][N]: calculate_gamma_TTT_3D_nested through gamma_3d_host's set-up on one
        thread (primordial and late term counts equal, as the reference sizes it)."""
        xvec, qt = (np.ascontiguousarray(a, dtype=np.float64) for a in (xvec, qt))
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        out = np.zeros((self.N, self.N))
        r = self.L.ref_gamma_3d(xvec.size, _p(xvec), qt.shape[1], _p(qt), prim.shape[0], _p(prim), float(dphi), _p(out))
        if r != 0:
            raise ValueError("ref_gamma_3d: the primordial term count must equal the late one")
        return out

    def gamma_transfer_pol(self, spec9, fsky_t, fsky_e, xvec, qtT, qtE, prim, dphi):
        """[4][N][Nprim]: calculate_gamma_2d's TTT, TTE, TEE, EEE with polarisation."""
        spec9 = np.ascontiguousarray(spec9, dtype=np.float64)
        xvec, qtT, qtE = (np.ascontiguousarray(a, dtype=np.float64) for a in (xvec, qtT, qtE))
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        self.L.ref_setup_pol_spectra(spec9.shape[1], _p(spec9), float(fsky_t), float(fsky_e))
        out = np.zeros((4, self.N, prim.shape[0]))
        self.L.ref_gamma_transfer_pol(xvec.size, _p(xvec), qtT.shape[1], _p(qtT), _p(qtE), prim.shape[0], _p(prim),
                                      float(dphi), _p(out))
        return out

    def prim_ortho(self, kmin, kmax_i, kmax, basis, prim):
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        N = prim.shape[0]
        out = np.empty(N * (N + 1) // 2)
        self.L.ref_prim_ortho(kmin, kmax_i, float(kmax), basis.shape[1], _p(basis), N, _p(prim), _p(out))
        return out

    def prim_eigen(self, kmin, kmax_i, kmax, basis, prim, shape):
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        N = prim.shape[0]
        a, n2 = np.empty(N), np.empty(1)
        kind, nterms, tab, c, sigma = _shape_args(shape)
        self.L.ref_prim_eigen(kmin, kmax_i, float(kmax), basis.shape[1], _p(basis), N, _p(prim), kind, nterms,
                              _p(tab), c[0], c[1], c[2], sigma, _p(a), _p(n2))
        return a, n2[0]

    def gamma_pol(self):
        """[4][N][N]: TTT, TTE, TEE, EEE from calculate_orthol over every pair."""
        out = np.zeros((4, self.N, self.N))
        self.L.ref_gamma_pol(_p(out))
        return out

    def orthol_pair(self, m, n):
        r = np.zeros(4)
        self.L.ref_orthol_pair(m, n, _p(r))
        return r[0]

    def gamma(self, nranks=8, npairs=0):
        out = np.zeros((self.N, self.N))
        n = self.L.ref_gamma(nranks, npairs, _p(out))
        return out, n

    def tetrapyd_walk(self, lmin, lmax, cap):
        pts = np.zeros((cap + 1, 3), dtype=np.int32)
        n = self.L.ref_tetrapyd_walk(lmin, lmax, cap, _p(pts))
        return pts[:min(n, cap + 1)], n

    def decompose(self, nthreads, lmin, lmax):
        out = np.zeros((nthreads, 4), dtype=np.int32)
        with quiet_stdout():
            self.L.ref_decompose(nthreads, lmin, lmax, _p(out))
        return out

    def modify_bispectrum(self, b, vec):
        b = np.array(b, dtype=np.float64, order="C", copy=True)
        vec = np.ascontiguousarray(vec, dtype=np.int32)
        self.L.ref_modify_bispectrum(b.shape[0], _p(vec), _p(b))
        return b

    def calculate_modes(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        beta = np.empty(self.N)
        with quiet_stdout():
            self.L.ref_calculate_modes(b.shape[0], _p(b), _p(beta))
        return beta

    def gamma_transfer(self, xvec, qt, prim, dphi):
        xvec = np.ascontiguousarray(xvec, dtype=np.float64)
        qt = np.ascontiguousarray(qt, dtype=np.float64)
        prim = np.ascontiguousarray(prim, dtype=np.int32)
        out = np.empty((self.N, prim.shape[0]))
        with quiet_stdout():
            self.L.ref_gamma_transfer(xvec.size, _p(xvec), qt.shape[1], _p(qt), prim.shape[0], _p(prim), float(dphi),
                                      _p(out))
        return out

    def project(self, shape, nthreads=8, max_points=0):
        beta = np.empty(self.N)
        if shape["kind"] == 0:
            tab = np.ascontiguousarray(shape["tab"], dtype=np.float64)
            args = (0, tab.shape[0], _p(tab), 0.0, 0.0, 0.0, 1.0)
        else:
            tab = None
            c = shape["c"]
            args = (1, 0, None, float(c[0]), float(c[1]), float(c[2]), float(shape["sigma"]))
        with quiet_stdout():
            self.L.ref_project(nthreads, *args, max_points, _p(beta))
        return beta


def basis_prune(gamma, faillist=(), steps=None):
    """Greedy basis pruning of basis_optimisation_mpi.c:184-337, restated with
    numpy.linalg.eigvalsh (LAPACK, upper triangle) standing in for
    LAPACKE_dsyevr(..., 'I', 'U', il = iu = 1).  The active modes are those not
    in faillist; Gamma is normalised as ortho[i][j] / (norm_i norm_j) (:184-190);
    each step computes the smallest eigenvalue of every leave-one-out minor
    (:256-281), removes the first maximiser (:287-312).  Returns (order,
    lambda_min) with the survivor last at lambda 1 (:326-343); `steps` stops
    early after that many removals (for large N), returning only those."""
    gamma = np.asarray(gamma, dtype=np.float64)
    N = gamma.shape[0]
    norm = np.sqrt(np.diag(gamma))
    failed = set(int(f) for f in faillist)
    lst = [i for i in range(N) if i not in failed]
    arr = gamma[np.ix_(lst, lst)] / np.outer(norm[lst], norm[lst])
    order, lams = [], []
    for n in range(len(lst) - 1, 0, -1):
        if steps is not None and len(order) == steps:
            return np.array(order), np.array(lams)
        vals = np.empty(n + 1)
        for m in range(n + 1):
            keep = np.r_[0:m, m + 1:n + 1]
            vals[m] = np.linalg.eigvalsh(arr[np.ix_(keep, keep)], UPLO="U")[0]
        index = int(np.argmax(vals))  # first maximum, as the strict '>' scan
        order.append(lst[index])
        lams.append(vals[index])
        del lst[index]
        arr = np.delete(np.delete(arr, index, 0), index, 1)
    order.append(lst[0])
    lams.append(1.0)
    return np.array(order), np.array(lams)


REF_PRUNE = os.path.join(HERE, "_ref", "basis_prune_ref")


def ref_basis_prune(gamma, faillist=()):
    """Run the reference's own basis_optimisation_mpi.c main() (compiled in
    place by `make -C oracle ref`, with its Gamma and fail-list reads redirected
    to temporary files and a Jacobi stand-in for MKL's dsyevr) and parse its
    printed elimination order: (order, lambda_min printed with %e)."""
    import tempfile
    gamma = np.ascontiguousarray(gamma, dtype=np.float64)
    N = gamma.shape[0]
    with tempfile.TemporaryDirectory() as d:
        gp = os.path.join(d, "gamma.unf")
        gamma.tofile(gp)
        env = dict(os.environ, MODAL_PRUNE_N=str(N), MODAL_PRUNE_GAMMA=gp)
        if len(faillist):
            fp = os.path.join(d, "fail.txt")
            with open(fp, "w") as f:
                f.write("\n".join(str(int(v)) for v in faillist) + "\n")
            env["MODAL_PRUNE_FAIL"] = fp
        out = subprocess.run([REF_PRUNE, "unused.ini"], env=env, check=True, capture_output=True, text=True).stdout
    lines = out.split("starting reduction\n", 1)[1].strip().splitlines()
    order = np.array([int(l.split("\t")[0]) for l in lines])
    lam = np.array([float(l.split("\t")[4]) for l in lines])
    return order, lam


# ------------------------------------------------------------------ data store

FILES_SO = os.path.join(HERE, "_ref", "libmodalfiles.so")


class RefFiles:
    """The reference's data-store sources (parameter.c, fixed_data.c, io.c,
    arrays.c, basis_functions.c) compiled in place into
    oracle/_ref/libmodalfiles.so, with the iniparser, GSL-spline and MPI
    stand-ins of refshim/files_glue.c.  One INI file at a time: the reference
    keeps its state in globals."""

    def __init__(self, path=FILES_SO):
        if not os.path.exists(path):
            if build_ref() is None:
                raise FileNotFoundError("reference checkout not present; oracle/_ref cannot be built")
        L = ctypes.CDLL(path)
        vp, i = ctypes.c_void_p, ctypes.c_int
        for name, args in [("files_init", [ctypes.c_char_p]), ("files_names", [ctypes.c_char_p, i]),
                           ("files_terms", [vp] * 6), ("files_spectra", [i, i, vp]), ("files_basis", [vp, vp]),
                           ("files_qtilde", [vp] * 6)]:
            fn = getattr(L, name)
            fn.restype, fn.argtypes = i, args
        self.L = L

    def load(self, ini_path):
        """initilise(ini): parameters and file names (parameter.c)."""
        with quiet_stdout():
            if self.L.files_init(ini_path.encode()) != 0:
                raise ValueError(f"initilise({ini_path}) failed")

    def names(self):
        buf = ctypes.create_string_buffer(1 << 16)
        if self.L.files_names(buf, len(buf)) != 0:
            raise ValueError("file-name buffer too small")
        return dict(line.split("=", 1) for line in buf.value.decode().splitlines())

    def terms(self, N, pol):
        """set_terms_prim + set_terms_late: {prim, ttt[, tte, tee, eee], pmax_prim, pmax_T, pmax_E}."""
        a = {k: np.zeros((N, 3), dtype=np.int32) for k in ("prim", "ttt", "tte", "tee", "eee")}
        pm = np.zeros(3, dtype=np.int32)
        with quiet_stdout():
            self.L.files_terms(*[_p(a[k]) for k in ("prim", "ttt", "tte", "tee", "eee")], _p(pm))
        if not pol:
            for k in ("tte", "tee", "eee"):
                del a[k]
        a.update(pmax_prim=int(pm[0]), pmax_T=int(pm[1]), pmax_E=int(pm[2]))
        return a

    def spectra(self, lmax, lens, tl):
        """load_cl + load_BN (+ load_lens, load_TL): [11][lmax+1] (see files_glue.c)."""
        out = np.zeros((11, lmax + 1))
        with quiet_stdout():
            if self.L.files_spectra(int(lens), int(tl), _p(out)) != 0:
                raise ValueError("spectrum tables rejected")
        return out

    def basis(self, Tsize, PT, Esize=0, PE=0):
        """create_basis_late: basis_late_T [Tsize][PT] (and basis_late_E)."""
        bt, be = np.zeros((Tsize, PT)), np.zeros((max(Esize, 1), max(PE, 1)))
        with quiet_stdout():
            self.L.files_basis(_p(bt), _p(be))
        return bt, (be if Esize else None)

    def qtilde(self, P, pol):
        """read_qtilde: {x, lvec_T, qt_T [P][lsize][xsize] (and E)}."""
        sizes = np.zeros(3, dtype=np.int32)
        with quiet_stdout():
            self.L.files_qtilde(_p(sizes), None, None, None, None, None)
        LT, LE, X = (int(v) for v in sizes)
        x, lt, qt = np.zeros(X), np.zeros(LT, dtype=np.int32), np.zeros((P, LT, X))
        le, qe = np.zeros(max(LE, 1), dtype=np.int32), np.zeros((P, max(LE, 1), X))
        self.L.files_qtilde(_p(sizes), _p(x), _p(lt), _p(qt), _p(le), _p(qe))
        out = {"x": x, "lvec_T": lt, "qt_T": qt}
        if pol:
            out.update(lvec_E=le, qt_E=qe)
        return out
