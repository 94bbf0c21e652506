"""Python host mirror of the C ABI in include/modal_gb300.h (ctypes).

The product is the shared library libmodal_gb300.so (CUDA kernels for
sm_103a behind a plain C ABI).  This module loads it, raises ModalError on
any non-zero status, and builds the synthetic workloads of the benchmark
configurations (synthetic spectrum, shifted Legendre basis, mode triples,
separable and Gaussian-bump shapes).  There is no CPU fallback: if the
library is missing, loading fails.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmodal_gb300.so")

PREC_FP64 = 0
PREC_SPLIT = 1
SHAPE_SEPARABLE = 0
SHAPE_BUMP = 1

STATUS = {0: "MODAL_OK", 1: "MODAL_ERR_ARG", 2: "MODAL_ERR_CUDA", 3: "MODAL_ERR_NOT_PD", 4: "MODAL_ERR_TIMEOUT",
          5: "MODAL_ERR_NOMEM", 6: "MODAL_ERR_STATE", 7: "MODAL_ERR_NOCONV"}

# Every entry point declared in include/modal_gb300.h.
EXPORTS = [
    "modal_ctx_create", "modal_ctx_destroy", "modal_last_error", "modal_ctx_stream", "modal_ctx_launches",
    "modal_ctx_sync", "modal_gl_nodes", "modal_legendre_table", "modal_basis_legendre", "modal_geometric",
    "modal_tetrapyd_count", "modal_set_basis", "modal_set_modes", "modal_set_gl", "modal_init_glint",
    "modal_get_mij", "modal_get_gl", "modal_gamma", "modal_gamma_partial", "modal_orthol_pair", "modal_orthogonalise",
    "modal_set_spectrum", "modal_project", "modal_alpha", "modal_ctx_profile", "modal_ctx_timer",
    "modal_ctx_timer_reset", "modal_gamma_fp64_noalloc", "modal_modify_bispectrum", "modal_calculate_modes",
    "modal_set_transfer", "modal_gamma_transfer", "modal_gamma_transfer_3d", "modal_project_gl", "modal_gamma_vjp", "modal_project_gl_vjp",
    "modal_alpha_gl", "modal_adjoint_residual", "modal_basis_prune", "modal_lambda_min",
    "modal_set_pca_floor", "modal_project_batch", "modal_ctx_captures", "modal_autotune", "modal_get_tuning",
    "modal_set_basis_e", "modal_set_modes_pol", "modal_gamma_pol", "modal_set_transfer_pol",
    "modal_gamma_transfer_pol", "modal_prim_points", "modal_prim_ortho", "modal_prim_eigen", "modal_set_ortho",
    "modal_eigh", "modal_gemm_f64", "modal_set_proj_kernel", "modal_get_proj_kernel",
]

TIMERS = {"gl": 0, "pl": 1, "mij": 2, "gamma": 3, "ortho": 4, "project": 5, "alpha": 6, "lift": 7, "adjoint": 8, "prune": 9,
          "eig_trd": 10, "eig_dc": 11, "eig_back": 12, "tc": 13,
          "eig_panel": 14}


class ModalError(RuntimeError):
    def __init__(self, status, msg):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


class CPolSpectra(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("cl_tt", "cl_te", "cl_ee", "beam_tt", "beam_te", "beam_ee",
                                                 "noise_tt", "noise_te", "noise_ee")] + \
               [("fsky_t", ctypes.c_double), ("fsky_e", ctypes.c_double)]


class CShape(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("nterms", ctypes.c_int), ("tab", ctypes.c_void_p),
                ("c", ctypes.c_double * 3), ("sigma", ctypes.c_double)]


_lib = None


def lib():
    """Load libmodal_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: run modal-cmb_gb300/build.py (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        vp, i, l, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double
        sig = {
            "modal_ctx_create": (i, [i, ctypes.POINTER(vp)]),
            "modal_ctx_destroy": (None, [vp]),
            "modal_last_error": (ctypes.c_char_p, []),
            "modal_ctx_stream": (vp, [vp]),
            "modal_ctx_launches": (l, [vp]),
            "modal_ctx_sync": (i, [vp]),
            "modal_gl_nodes": (i, [i, vp, vp]),
            "modal_legendre_table": (i, [i, i, vp, vp]),
            "modal_basis_legendre": (i, [i, i, d, d, vp, vp]),
            "modal_geometric": (i, [l, vp, vp]),
            "modal_tetrapyd_count": (i, [i, i, ctypes.POINTER(l)]),
            "modal_set_basis": (i, [vp, i, i, i, vp]),
            "modal_set_modes": (i, [vp, i, vp]),
            "modal_set_gl": (i, [vp, i, vp, vp]),
            "modal_init_glint": (i, [vp]),
            "modal_get_mij": (i, [vp, vp]),
            "modal_get_gl": (i, [vp, ctypes.POINTER(i), vp, vp]),
            "modal_gamma": (i, [vp, i, vp]),
            "modal_gamma_partial": (i, [vp, i, i, i, vp]),
            "modal_orthol_pair": (i, [vp, i, i, vp]),
            "modal_orthogonalise": (i, [vp, vp, i, vp, vp, ctypes.POINTER(i), ctypes.POINTER(i)]),
            "modal_set_spectrum": (i, [vp, vp]),
            "modal_project": (i, [vp, i, vp, i, vp]),
            "modal_alpha": (i, [vp, i, vp, vp, vp]),
            "modal_ctx_profile": (i, [vp, i]),
            "modal_ctx_timer": (i, [vp, i, ctypes.POINTER(d), ctypes.POINTER(l)]),
            "modal_ctx_timer_reset": (i, [vp]),
            "modal_gamma_fp64_noalloc": (i, [i, i, i, vp, i, vp, i, vp, vp, vp, vp]),
            "modal_modify_bispectrum": (i, [i, vp, vp, vp, vp, vp]),
            "modal_calculate_modes": (i, [vp, i, vp, vp]),
            "modal_set_transfer": (i, [vp, i, i, vp, vp, i, vp]),
            "modal_gamma_transfer": (i, [vp, d, vp]),
            "modal_gamma_transfer_3d": (i, [vp, d, vp]),
            "modal_set_ortho": (i, [vp, vp, vp]),
            "modal_project_gl": (i, [vp, i, vp, vp, vp]),
            "modal_gamma_vjp": (i, [vp, vp, vp]),
            "modal_project_gl_vjp": (i, [vp, i, vp, vp, vp]),
            "modal_alpha_gl": (i, [vp, i, vp, vp, vp, vp]),
            "modal_adjoint_residual": (i, [vp, i, vp, ctypes.POINTER(d), vp]),
            "modal_basis_prune": (i, [vp, i, vp, i, vp, vp, vp]),
            "modal_lambda_min": (i, [vp, ctypes.POINTER(d), vp, vp]),
            "modal_set_pca_floor": (i, [vp, d]),
            "modal_set_proj_kernel": (i, [vp, i]),
            "modal_get_proj_kernel": (i, [vp, vp]),
            "modal_eigh": (i, [vp, i, vp, vp, vp]),
            "modal_gemm_f64": (i, [vp, i, i, i, d, vp, i, vp, i, d, vp, i]),
            "modal_project_batch": (i, [vp, i, vp, i, vp]),
            "modal_ctx_captures": (l, [vp]),
            "modal_autotune": (i, [vp, ctypes.c_char_p]),
            "modal_get_tuning": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]),
            "modal_set_basis_e": (i, [vp, i, i, i, vp]),
            "modal_set_modes_pol": (i, [vp, vp, vp, vp]),
            "modal_gamma_pol": (i, [vp, vp, vp, vp]),
            "modal_set_transfer_pol": (i, [vp, vp, vp]),
            "modal_gamma_transfer_pol": (i, [vp, d, vp, vp, vp]),
            "modal_prim_points": (i, [i, i, ctypes.POINTER(l), vp]),
            "modal_prim_ortho": (i, [vp, i, i, d, i, vp, i, vp, vp]),
            "modal_prim_eigen": (i, [vp, i, i, d, i, vp, i, vp, i, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(status):
    if status != 0:
        raise ModalError(status, lib().modal_last_error().decode(errors="replace"))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---------------------------------------------------------------- primitives

def gl_nodes(n):
    """Gauss-Legendre nodes/weights on the GPU (asy() layout)."""
    x = np.empty(n)
    w = np.empty(n)
    _check(lib().modal_gl_nodes(n, _ptr(x), _ptr(w)))
    return x, w


def legendre_table(mu, lmax):
    """[nmu][lmax+1] table (2l+1)^{2/3} P_l(mu_k) on the GPU."""
    mu = _f64(mu)
    out = np.empty((mu.size, lmax + 1))
    _check(lib().modal_legendre_table(mu.size, lmax, _ptr(mu), _ptr(out)))
    return out


def basis_legendre(values, pmax, vmin, vmax):
    values = _f64(values)
    out = np.empty((values.size, pmax + 1))
    _check(lib().modal_basis_legendre(values.size, pmax, float(vmin), float(vmax), _ptr(values), _ptr(out)))
    return out


def geometric(pts):
    pts = np.ascontiguousarray(pts, dtype=np.int32).reshape(-1, 3)
    out = np.empty(pts.shape[0])
    _check(lib().modal_geometric(pts.shape[0], _ptr(pts), _ptr(out)))
    return out


def tetrapyd_count(lmin, lmax):
    n = ctypes.c_long()
    _check(lib().modal_tetrapyd_count(lmin, lmax, ctypes.byref(n)))
    return n.value


def modify_bispectrum(b, vec, cl, beam=None, noise=None):
    """modify_bispectrum on the GPU; returns the modified copy of b[size][size][size]."""
    b = np.array(b, dtype=np.float64, order="C", copy=True)
    size = b.shape[0]
    vec = np.ascontiguousarray(vec, dtype=np.int32)
    cl = _f64(cl)
    beam = np.ones(size) if beam is None else _f64(beam)
    noise = np.zeros(size) if noise is None else _f64(noise)
    _check(lib().modal_modify_bispectrum(size, _ptr(vec), _ptr(cl), _ptr(beam), _ptr(noise), _ptr(b)))
    return b


def shapes_to_c(shapes):
    """List of shape dicts -> (ctypes array, keep-alive list)."""
    arr = (CShape * len(shapes))()
    keep = []
    for s, sh in enumerate(shapes):
        arr[s].kind = sh["kind"]
        if sh["kind"] == SHAPE_SEPARABLE:
            tab = _f64(sh["tab"])
            keep.append(tab)
            arr[s].nterms = tab.shape[0]
            arr[s].tab = tab.ctypes.data
        else:
            arr[s].c[0], arr[s].c[1], arr[s].c[2] = (float(v) for v in sh["c"])
            arr[s].sigma = float(sh["sigma"])
    return arr, keep


class Context:
    """One GPU context (device buffers + one CUDA stream)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().modal_ctx_create(device, ctypes.byref(h)))
        self.h = h
        self.N = self.P = self.lmin = self.lmax = None

    def close(self):
        if self.h:
            lib().modal_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return lib().modal_ctx_stream(self.h)

    @property
    def launches(self):
        return lib().modal_ctx_launches(self.h)

    def sync(self):
        _check(lib().modal_ctx_sync(self.h))

    def profile(self, enable=True):
        _check(lib().modal_ctx_profile(self.h, int(enable)))

    def timer(self, name):
        """(summed ms, count) of a stage's device time since the last reset."""
        ms, n = ctypes.c_double(), ctypes.c_long()
        _check(lib().modal_ctx_timer(self.h, TIMERS[name], ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def timer_reset(self):
        _check(lib().modal_ctx_timer_reset(self.h))

    def set_basis(self, lmin, lmax, q):
        q = _f64(q)
        assert q.shape[0] == lmax - lmin + 1
        _check(lib().modal_set_basis(self.h, lmin, lmax, q.shape[1], _ptr(q)))
        self.lmin, self.lmax, self.P = lmin, lmax, q.shape[1]

    def set_modes(self, triples):
        t = np.ascontiguousarray(triples, dtype=np.int32).reshape(-1, 3)
        _check(lib().modal_set_modes(self.h, t.shape[0], _ptr(t)))
        self.N = t.shape[0]

    def set_gl(self, nodes, weights):
        nodes, weights = _f64(nodes), _f64(weights)
        _check(lib().modal_set_gl(self.h, nodes.size, _ptr(nodes), _ptr(weights)))

    def init_glint(self):
        _check(lib().modal_init_glint(self.h))

    def get_gl(self):
        n = ctypes.c_int()
        _check(lib().modal_get_gl(self.h, ctypes.byref(n), None, None))
        x, w = np.empty(n.value), np.empty(n.value)
        _check(lib().modal_get_gl(self.h, ctypes.byref(n), _ptr(x), _ptr(w)))
        return x, w

    def get_mij(self):
        n = ctypes.c_int()
        _check(lib().modal_get_gl(self.h, ctypes.byref(n), None, None))
        out = np.empty((self.P, self.P, n.value))
        _check(lib().modal_get_mij(self.h, _ptr(out)))
        return out

    def gamma(self, prec=PREC_FP64, download=True, out=None):
        """Gamma [N][N]; `out` may be a caller array (e.g. a view of pinned memory)."""
        if out is None:
            out = np.empty((self.N, self.N)) if (download and self.N) else None
        else:
            assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.N * self.N
        _check(lib().modal_gamma(self.h, prec, _ptr(out)))
        return out

    def gamma_partial(self, prec, mu_begin, mu_end):
        """Gamma over the quadrature nodes mu_begin..mu_end-1 only (a shard of the
        sum over mu; partials over a partition of the nodes add up to Gamma)."""
        out = np.empty((self.N, self.N))
        _check(lib().modal_gamma_partial(self.h, prec, mu_begin, mu_end, _ptr(out)))
        return out

    def orthol_pair(self, m, n, all_four=False):
        r = np.zeros(4)
        _check(lib().modal_orthol_pair(self.h, m, n, _ptr(r)))
        return r if all_four else r[0]

    def set_basis_e(self, lmin, lmax, qe):
        qe = _f64(qe)
        assert qe.shape[0] == lmax - lmin + 1
        _check(lib().modal_set_basis_e(self.h, lmin, lmax, qe.shape[1], _ptr(qe)))

    def set_modes_pol(self, tte, tee, eee):
        t = [np.ascontiguousarray(x, dtype=np.int32).reshape(-1, 3) for x in (tte, tee, eee)]
        _check(lib().modal_set_modes_pol(self.h, _ptr(t[0]), _ptr(t[1]), _ptr(t[2])))

    def gamma_pol(self):
        outs = [np.empty((self.N, self.N)) for _ in range(3)]
        _check(lib().modal_gamma_pol(self.h, _ptr(outs[0]), _ptr(outs[1]), _ptr(outs[2])))
        return tuple(outs)

    def orthogonalise(self, gamma=None, pca_flag=1, download=True, out=None):
        """(orthol, lambdal, branch, rank); `out` = (orthol, lambdal) caller arrays."""
        g = None if gamma is None else _f64(gamma)
        if out is not None:
            o, lam = out
        else:
            o = np.empty((self.N, self.N)) if download else None
            lam = np.empty((self.N, self.N)) if download else None
        br, rk = ctypes.c_int(), ctypes.c_int()
        _check(lib().modal_orthogonalise(self.h, _ptr(g), pca_flag, _ptr(o), _ptr(lam), ctypes.byref(br),
                                         ctypes.byref(rk)))
        return o, lam, br.value, rk.value

    def set_pca_floor(self, floor):
        _check(lib().modal_set_pca_floor(self.h, float(floor)))

    def set_proj_kernel(self, tensor_cores):
        """FP32 projection kernel: True = tcgen05 tensor cores (P <= 32), False = CUDA cores."""
        _check(lib().modal_set_proj_kernel(self.h, 1 if tensor_cores else 0))

    def proj_kernel(self):
        """True when the FP32 projection of the current basis runs on the tensor cores."""
        v = ctypes.c_int()
        _check(lib().modal_get_proj_kernel(self.h, ctypes.byref(v)))
        return bool(v.value)

    def gemm_f64(self, A, B, transA=False, transB=False, alpha=1.0, beta=0.0, C=None, slices=8):
        """alpha op(A) op(B) + beta C in FP64 accuracy on the tensor cores
        (modal_gemm_f64: exact 7-bit integer slices of the operands)."""
        A, B = _f64(A), _f64(B)
        M = A.shape[1] if transA else A.shape[0]
        K = A.shape[0] if transA else A.shape[1]
        N = B.shape[0] if transB else B.shape[1]
        assert (B.shape[1] if transB else B.shape[0]) == K
        C = np.zeros((M, N)) if C is None else _f64(C).copy()
        _check(lib().modal_gemm_f64(self.h, M, N, K, float(alpha), _ptr(A), int(transA), _ptr(B), int(transB),
                                    float(beta), _ptr(C), int(slices)))
        return C

    def eigh(self, a, vectors=True):
        """(w ascending, v with eigenvectors as rows or None) of the symmetric matrix a
        (modal_eigh: the library's own FP64 eigensolver on the GPU)."""
        a = _f64(a)
        n = a.shape[0]
        assert a.shape == (n, n)
        w = np.empty(n)
        v = np.empty((n, n)) if vectors else None
        _check(lib().modal_eigh(self.h, n, _ptr(a), _ptr(w), _ptr(v)))
        return w, v

    def set_spectrum(self, cl):
        cl = _f64(cl)
        assert cl.size >= self.lmax + 1
        _check(lib().modal_set_spectrum(self.h, _ptr(cl)))

    def project(self, shapes, prec=PREC_FP64, download=True):
        arr, keep = shapes_to_c(shapes)
        out = np.empty((len(shapes), self.N)) if download else None
        _check(lib().modal_project(self.h, len(shapes), ctypes.cast(arr, ctypes.c_void_p), prec, _ptr(out)))
        del keep
        return out

    def project_batch(self, shapes, prec=PREC_FP64):
        """beta [S][N] through the captured-graph batch path."""
        arr, keep = shapes_to_c(shapes)
        out = np.empty((len(shapes), self.N))
        _check(lib().modal_project_batch(self.h, len(shapes), ctypes.cast(arr, ctypes.c_void_p), prec, _ptr(out)))
        del keep
        return out

    @property
    def captures(self):
        return lib().modal_ctx_captures(self.h)

    def autotune(self, cache_path=None):
        _check(lib().modal_autotune(self.h, None if cache_path is None else os.fsencode(cache_path)))
        return self.tuning()

    def tuning(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().modal_get_tuning(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"proj_sg": a.value, "proj_cpb": b.value, "gamma_kc": c.value, "proj_tc": int(self.proj_kernel())}

    def set_transfer(self, xvec, qtilde, prim):
        xvec = _f64(xvec)
        qt = _f64(qtilde)
        prim = np.ascontiguousarray(prim, dtype=np.int32).reshape(-1, 3)
        _check(lib().modal_set_transfer(self.h, qt.shape[1], xvec.size, _ptr(xvec), _ptr(qt), prim.shape[0], _ptr(prim)))
        self.Nprim = prim.shape[0]

    def gamma_transfer(self, deltaphi):
        out = np.empty((self.N, self.Nprim))
        _check(lib().modal_gamma_transfer(self.h, float(deltaphi), _ptr(out)))
        return out

    def gamma_transfer_3d(self, deltaphi):
        """[N][Nprim] 3D transfer Gamma (tetrapyd sum of the radial integrals)."""
        out = np.empty((self.N, self.Nprim))
        _check(lib().modal_gamma_transfer_3d(self.h, float(deltaphi), _ptr(out)))
        return out

    def set_transfer_pol(self, qtilde_e, spec9, fsky_t, fsky_e):
        """spec9: cl_tt, cl_te, cl_ee, beam_tt, beam_te, beam_ee, noise_tt, noise_te, noise_ee over l."""
        qe = _f64(qtilde_e)
        arrs = [_f64(a) for a in spec9]
        sp = CPolSpectra(*[a.ctypes.data for a in arrs], float(fsky_t), float(fsky_e))
        _check(lib().modal_set_transfer_pol(self.h, _ptr(qe), ctypes.byref(sp)))

    def gamma_transfer_pol(self, deltaphi):
        outs = [np.empty((self.N, self.Nprim)) for _ in range(3)]
        _check(lib().modal_gamma_transfer_pol(self.h, float(deltaphi), _ptr(outs[0]), _ptr(outs[1]), _ptr(outs[2])))
        return tuple(outs)

    def prim_ortho(self, kmin, kmax_i, kmax, basis, prim):
        """Packed upper triangle [N(N+1)/2] of the primordial k-grid Gram matrix."""
        basis = _f64(basis)
        prim = np.ascontiguousarray(prim, dtype=np.int32).reshape(-1, 3)
        N = prim.shape[0]
        out = np.empty(N * (N + 1) // 2)
        _check(lib().modal_prim_ortho(self.h, kmin, kmax_i, float(kmax), basis.shape[1], _ptr(basis), N, _ptr(prim),
                                      _ptr(out)))
        return out

    def prim_eigen(self, kmin, kmax_i, kmax, basis, prim, shapes):
        """(alpha [S][N], <S,S> [S]) of primordial shapes on the k-grid."""
        basis = _f64(basis)
        prim = np.ascontiguousarray(prim, dtype=np.int32).reshape(-1, 3)
        arr, keep = shapes_to_c(shapes)
        a, n2 = np.empty((len(shapes), prim.shape[0])), np.empty(len(shapes))
        _check(lib().modal_prim_eigen(self.h, kmin, kmax_i, float(kmax), basis.shape[1], _ptr(basis), prim.shape[0],
                                      _ptr(prim), len(shapes), ctypes.cast(arr, ctypes.c_void_p), _ptr(a), _ptr(n2)))
        del keep
        return a, n2

    def calculate_modes(self, b):
        b = _f64(b)
        out = np.empty(self.N)
        _check(lib().modal_calculate_modes(self.h, b.shape[0], _ptr(b), _ptr(out)))
        return out

    # ---- adjoint (gradients with respect to q[L][P])

    def project_gl(self, shapes):
        """(beta [S][N], <S,S> [S]) in Gamma's Gauss-Legendre inner product."""
        arr, keep = shapes_to_c(shapes)
        beta, n2 = np.empty((len(shapes), self.N)), np.empty(len(shapes))
        _check(lib().modal_project_gl(self.h, len(shapes), ctypes.cast(arr, ctypes.c_void_p), _ptr(beta), _ptr(n2)))
        del keep
        return beta, n2

    def gamma_vjp(self, dL_dgamma):
        g = _f64(dL_dgamma)
        out = np.empty((self.lmax - self.lmin + 1, self.P))
        _check(lib().modal_gamma_vjp(self.h, _ptr(g), _ptr(out)))
        return out

    def project_gl_vjp(self, shapes, dL_dbeta):
        arr, keep = shapes_to_c(shapes)
        g = _f64(dL_dbeta)
        out = np.empty((self.lmax - self.lmin + 1, self.P))
        _check(lib().modal_project_gl_vjp(self.h, len(shapes), ctypes.cast(arr, ctypes.c_void_p), _ptr(g), _ptr(out)))
        del keep
        return out

    def alpha_gl(self, shapes, dL_dalpha=None):
        """alpha [S][N]; with dL_dalpha also dL/dq [L][P]."""
        arr, keep = shapes_to_c(shapes)
        a = np.empty((len(shapes), self.N))
        g = None if dL_dalpha is None else _f64(dL_dalpha)
        out = None if g is None else np.empty((self.lmax - self.lmin + 1, self.P))
        _check(lib().modal_alpha_gl(self.h, len(shapes), ctypes.cast(arr, ctypes.c_void_p), _ptr(a), _ptr(g), _ptr(out)))
        del keep
        return a if g is None else (a, out)

    def adjoint_residual(self, shapes, grad=True):
        """(J, dJ/dq [L][P] or None): mean relative squared projection residual."""
        arr, keep = shapes_to_c(shapes)
        J = ctypes.c_double()
        out = np.empty((self.lmax - self.lmin + 1, self.P)) if grad else None
        _check(lib().modal_adjoint_residual(self.h, len(shapes), ctypes.cast(arr, ctypes.c_void_p), ctypes.byref(J),
                                            _ptr(out)))
        del keep
        return J.value, out

    def basis_prune(self, gamma=None, faillist=(), N=None):
        """(order, lambda_min): greedy pruning order of the active modes."""
        g = None if gamma is None else _f64(gamma)
        N = g.shape[0] if g is not None else (N or self.N)
        fl = np.ascontiguousarray(faillist, dtype=np.int32)
        n = N - fl.size
        order, lam = np.empty(max(n, 1), dtype=np.int32), np.empty(max(n, 1))
        _check(lib().modal_basis_prune(self.h, N, _ptr(g), fl.size, _ptr(fl) if fl.size else None, _ptr(order),
                                       _ptr(lam)))
        return order[:n], lam[:n]

    def lambda_min(self, grad=False):
        """(lambda_min, eigenvector, dlambda/dq or None) of the normalised device Gamma."""
        lam = ctypes.c_double()
        v = np.empty(self.N)
        out = np.empty((self.lmax - self.lmin + 1, self.P)) if grad else None
        _check(lib().modal_lambda_min(self.h, ctypes.byref(lam), _ptr(v), _ptr(out)))
        return lam.value, v, out

    def set_ortho(self, orthol, lambdal):
        """Load orthol/lambdal [N][N] (e.g. read from the orthol/lambdal files) for alpha."""
        o, lam = _f64(orthol), _f64(lambdal)
        assert o.shape == lam.shape == (self.N, self.N)
        _check(lib().modal_set_ortho(self.h, _ptr(o), _ptr(lam)))

    def alpha(self, S, beta=None, download=True):
        b = None if beta is None else _f64(beta)
        a = np.empty((S, self.N)) if download else None
        m = np.empty((S, self.N)) if download else None
        _check(lib().modal_alpha(self.h, S, _ptr(b), _ptr(a), _ptr(m)))
        return a, m


# ----------------------------------------------------------- synthetic inputs

def prim_points(kmin, kmax_i):
    """[npts][3] points of the primordial k-grid tetrapyd, enumerated on the GPU."""
    n = ctypes.c_long()
    _check(lib().modal_prim_points(kmin, kmax_i, ctypes.byref(n), None))
    pts = np.empty((n.value, 3), dtype=np.int32)
    _check(lib().modal_prim_points(kmin, kmax_i, ctypes.byref(n), _ptr(pts)))
    return pts


def synthetic_cl(lmax):
    """C_l = 1e3/(l(l+1)) exp(-(l/1500)^2) + 1e-4 (noise, beam 1); l < 2 set to 1."""
    l = np.arange(lmax + 1, dtype=np.float64)
    cl = np.ones(lmax + 1)
    ll = l[2:]
    cl[2:] = 1e3 / (ll * (ll + 1.0)) * np.exp(-(ll / 1500.0) ** 2) + 1e-4
    return cl


def legendre_q(lmin, lmax, P):
    """Shifted Legendre basis q_p(l) = P_p(2(l-lmin)/(lmax-lmin) - 1), [L][P]
    (basis_functions_legendre with min=lmin, max=lmax; numpy restatement used
    only to build inputs)."""
    l = np.arange(lmin, lmax + 1, dtype=np.float64)
    x = (l - lmin) / (lmax - lmin)
    q = np.zeros((l.size, P))
    q[:, 0] = 1.0
    if P > 1:
        q[:, 1] = 2.0 * x - 1.0
    for j in range(2, P):
        q[:, j] = ((2.0 * j - 1.0) * q[:, 1] * q[:, j - 1] - (j - 1.0) * q[:, j - 2]) / j
    return q


def weighted_q(q, cl, lmin):
    """q~_p(l) = q_p(l) (2l+1)^{1/6} / sqrt(C_l): with the (2l+1)^{2/3} of the
    P_l table this gives A_pp'(mu) = sum_l (2l+1) P_l(mu) q_p q_p' / C_l."""
    l = np.arange(lmin, lmin + q.shape[0], dtype=np.float64)
    return q * ((2.0 * l + 1.0) ** (1.0 / 6.0) / np.sqrt(cl[lmin:lmin + q.shape[0]]))[:, None]


def mode_triples(P):
    """All p <= r <= s < P, in the order of set_terms_late case 2
    (fixed_data.c:362-418: increasing total p+r+s), keeping entries < P."""
    want = P * (P + 1) * (P + 2) // 6
    out = []
    i = j = k = s = 0
    while len(out) < want:
        if k < P:
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


def separable_shapes(lmax, S, seed, tmin=1, tmax=2):
    """S seeded shapes S = sym sum_t l1^a l2^b l3^c, a,b,c ~ U[-2,0], T ~ U{tmin..tmax}."""
    rng = np.random.default_rng(seed)
    l = np.arange(lmax + 1, dtype=np.float64)
    l[0] = 1.0  # l = 0,1 never reached (lmin >= 2)
    out = []
    for _ in range(S):
        T = int(rng.integers(tmin, tmax + 1))
        ex = rng.uniform(-2.0, 0.0, size=(T, 3))
        tab = np.empty((T, 3, lmax + 1))
        for t in range(T):
            for a in range(3):
                tab[t, a] = l ** ex[t, a]
        out.append({"kind": SHAPE_SEPARABLE, "tab": tab, "exponents": ex})
    return out


def pol_workload(lmaxT, lmaxE, lminE, PT, PE):
    """Polarised case: T basis on 2..lmaxT, E basis on lminE..lmaxE with its own
    weight, and the first N = C(PT+2, 3) triples of each family in the
    find_perm_late_XXX conventions (TTE: T,T,E; TEE: T,E,E; EEE)."""
    cl = synthetic_cl(max(lmaxT, lmaxE))
    qT = weighted_q(legendre_q(2, lmaxT, PT), cl, 2)
    qE = weighted_q(legendre_q(lminE, lmaxE, PE), cl * 2.0, lminE)
    ttt = mode_triples(PT)
    N = len(ttt)
    tte = np.array([(p, r, s) for p in range(PT) for r in range(p, PT) for s in range(PE)][:N], dtype=np.int32)
    tee = np.array([(t, a, b) for t in range(PT) for a in range(PE) for b in range(a, PE)][:N], dtype=np.int32)
    eee = mode_triples(PE)[:N]
    return cl, qT, qE, ttt, tte, tee, eee


def transfer_workload(lmax, Pp, xsize):
    """Radial grid x in [1000, 12000] and smooth synthetic transfer functions
    q~_p(l, x) [xsize][Pp][lmax+1] for the late x primordial Gamma."""
    xvec = np.linspace(1000.0, 12000.0, xsize)
    l = np.arange(lmax + 1.0)
    p = np.arange(Pp)[:, None]
    qt = np.stack([np.cos((p + 1) * x / 4000.0) * np.sin(0.1 * l * (1 + p) + x / 3000.0) / (1.0 + l) for x in xvec])
    return xvec, qt


def prim_workload(kmax_i, Pp):
    """Primordial k-grid case: cosine basis on grid indices 0..kmax_i, all
    p <= r <= s < Pp triples, one separable and one bump shape."""
    x = np.arange(kmax_i + 1) / kmax_i
    basis = np.stack([np.cos(np.pi * p * x) + 0.1 * p * x for p in range(Pp)], axis=1)
    shapes = separable_shapes(kmax_i, 1, 3, 1, 2) + bump_shapes(1, 4)
    for sh in shapes:  # index 0 unused with kmin = 1
        if sh["kind"] == SHAPE_SEPARABLE:
            sh["tab"][:, :, 0] = 0.0
    return basis, mode_triples(Pp), shapes


def bspline_matrix(lmin, lmax, nb=64, degree=3):
    """[L][nb] clamped uniform B-splines of the given degree on [lmin, lmax]
    (Cox-de Boor recursion; input builder for the basis-optimisation workload)."""
    l = np.arange(lmin, lmax + 1, dtype=np.float64)
    x = (l - lmin) / (lmax - lmin)
    inner = np.linspace(0.0, 1.0, nb - degree + 1)
    t = np.concatenate([np.zeros(degree), inner, np.ones(degree)])
    B = np.zeros((x.size, len(t) - 1))
    for i in range(len(t) - 1):
        B[:, i] = (x >= t[i]) & (x < t[i + 1])
    B[x >= 1.0, nb - 1] = 1.0  # right end belongs to the last non-empty span
    for k in range(1, degree + 1):
        Bn = np.zeros((x.size, len(t) - 1 - k))
        for i in range(len(t) - 1 - k):
            a = t[i + k] - t[i]
            b = t[i + k + 1] - t[i + 1]
            left = (x - t[i]) / a * B[:, i] if a > 0 else 0.0
            right = (t[i + k + 1] - x) / b * B[:, i + 1] if b > 0 else 0.0
            Bn[:, i] = left + right
        B = Bn
    return B


def bspline_workload(lmax=1000, nfunc=12, nb=64, seed=0, lmin=2):
    """Basis-optimisation workload: q_p = sum_j C[p][j] B_j(l) with a seeded
    [nfunc][nb] FP64 coefficient matrix.  Returns (C, Bw, triples, cl) where
    Bw[l][j] = B_j(l) (2l+1)^{1/6}/sqrt(C_l), so that q~ = Bw C^T."""
    cl = synthetic_cl(lmax)
    B = bspline_matrix(lmin, lmax, nb)
    Bw = weighted_q(B, cl, lmin)
    C = np.random.default_rng(seed).standard_normal((nfunc, nb))
    return C, Bw, mode_triples(nfunc), cl


def bump_shapes(S, seed):
    """S seeded Gaussian bumps, centre ~ Dirichlet(1,1,1), sigma ~ U[0.05,0.3]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(S):
        c = rng.dirichlet([1.0, 1.0, 1.0])
        out.append({"kind": SHAPE_BUMP, "c": c, "sigma": float(rng.uniform(0.05, 0.3))})
    return out


# The benchmark configurations (lmin = 2 everywhere).
CONFIGS = {
    "cfg1": dict(lmax=500, P=10, shapes=("sep", 4, 1, 2)),
    "cfg2": dict(lmax=2000, P=30, shapes=("sep", 16, 1, 2)),
    "cfg3": dict(lmax=2000, P=30, shapes=("mix", 256, 1, 4)),
    "cfg4": dict(lmax=1000, P=12, shapes=("sep", 32, 1, 2), basis="bspline64"),
    "cfg5": dict(lmax=2500, P=40, shapes=("mix", 512, 1, 4)),
    # mid-size case for kernel captures: operands larger than L2, a few GB at most
    "prof": dict(lmax=1000, P=20, shapes=("sep", 4, 1, 2)),
}


def mu_shard(nmu, rank, world):
    """[begin, end) of the quadrature nodes that rank `rank` of `world` sums over:
    the balanced split the reference uses for its pair loop (ortho_late_mpi.c:
    240-255), the first nmu % world ranks taking one node more."""
    if not (0 <= rank < world) or nmu < world:
        raise ValueError(f"mu_shard: rank {rank} of {world} for {nmu} nodes")
    base, extra = divmod(nmu, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def workload(lmax, P, lmin=2):
    """(q~ [L][P], triples [N][3], cl [lmax+1]) for a shifted-Legendre config."""
    cl = synthetic_cl(lmax)
    q = weighted_q(legendre_q(lmin, lmax, P), cl, lmin)
    return q, mode_triples(P), cl


def config_shapes(lmax, spec, seed=0):
    kind, S, tmin, tmax = spec
    if kind == "sep":
        return separable_shapes(lmax, S, seed, tmin, tmax)
    half = S // 2
    return separable_shapes(lmax, half, seed, tmin, tmax) + bump_shapes(S - half, seed + 1)
