"""FP64 reference for the adjoint tests: the forward quantities that the
library's hand-written adjoint kernels differentiate, written as plain torch
float64 operations so that torch autograd gives an independent reference
gradient.  Test infrastructure only.

  pl[l][k]  = (2l+1)^{2/3} P_l(mu_k)                       (gl_Pl of orthogonalisation_late.c)
  M[k][p][q] = sum_l pl q_p q_q,  Gamma = sum_k w_k/(48 pi) perm3(M[k][m_a][n_b])
  B[k][e][q] = sum_l pl f~_e q_q,  beta_sn = sum_k w_k/(48 pi) sum_t perm3(B[k][(s,t,a)][n_b])
  <S,S>      = sum_k w_k/(48 pi) sum_{t,t'} perm3(<f~_(s,t,a), f~_(s,t',b)>_k)
  J          = mean_s (<S,S> - beta_s . Gamma^{-1} beta_s) / <S,S>
with f~ = w_l f, w_l = (2l+1)^{1/6}/sqrt(C_l) (calculate_mode_3D.c:53-62).
"""
import math

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

INV48PI = 1.0 / (48.0 * math.pi)
PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


def pl_table(mu, lmin, lmax):
    """[L][K] (2l+1)^{2/3} P_l(mu_k) for l = lmin..lmax (three-term recurrence)."""
    mu = np.asarray(mu, dtype=np.float64)
    P = np.empty((lmax + 1, mu.size))
    P[0] = 1.0
    if lmax >= 1:
        P[1] = mu
    for l in range(1, lmax):
        P[l + 1] = ((2 * l + 1) * mu * P[l] - l * P[l - 1]) / (l + 1)
    l = np.arange(lmax + 1, dtype=np.float64)
    return (P * ((2 * l + 1) ** (2.0 / 3.0))[:, None])[lmin:]


def leg_weight(cl, lmin, lmax):
    l = np.arange(lmin, lmax + 1, dtype=np.float64)
    w = (2 * l + 1) ** (1.0 / 6.0) / np.sqrt(cl[lmin:lmax + 1])
    w[l < 2] = 0.0
    return w


def _perm_rows(A, ri, ci):
    """sum over the 6 permutations: out[k][i][j] = perm3(A[k][ri[i][a]][ci[j][b]])."""
    acc = 0.0
    for s in PERMS:
        acc = acc + (A[:, ri[:, 0, None], ci[None, :, s[0]]] * A[:, ri[:, 1, None], ci[None, :, s[1]]] *
                     A[:, ri[:, 2, None], ci[None, :, s[2]]])
    return acc


def _chunk(A, wc, ri, ci):
    return torch.einsum("k,kmn->mn", wc, _perm_rows(A, ri, ci))


def quad_perm(A, w, ri, ci, chunk=64):
    """sum_k w_k/(48 pi) perm3(A[k][ri[i][a]][ci[j][b]]) -> [len(ri)][len(ci)], chunked over k
    with recomputation in the backward pass to bound memory."""
    out = None
    for k0 in range(0, A.shape[0], chunk):
        part = checkpoint(_chunk, A[k0:k0 + chunk], w[k0:k0 + chunk] * INV48PI, ri, ci, use_reentrant=False)
        out = part if out is None else out + part
    return out


def shape_legs(shapes, cl, lmin, lmax):
    """([E][L] weighted legs, [(first leg, terms)] per shape) for separable shapes."""
    wl = leg_weight(cl, lmin, lmax)
    legs, info, e = [], [], 0
    for sh in shapes:
        tab = np.asarray(sh["tab"], dtype=np.float64)
        T = tab.shape[0]
        info.append((e, T))
        for t in range(T):
            for a in range(3):
                legs.append(wl * tab[t, a, lmin:lmax + 1])
        e += 3 * T
    return np.array(legs), info


class Problem:
    """Fixed inputs of one objective: Legendre table, weights, triples, shape legs."""

    def __init__(self, mu, w, lmin, lmax, triples, cl, shapes, device="cpu"):
        dt = dict(dtype=torch.float64, device=device)
        self.pl = torch.tensor(pl_table(mu, lmin, lmax), **dt)
        self.w = torch.tensor(np.asarray(w, dtype=np.float64), **dt)
        self.tri = torch.tensor(np.asarray(triples, dtype=np.int64), device=device)
        self.device = device
        if shapes:
            legs, self.info = shape_legs(shapes, cl, lmin, lmax)
            self.legs = torch.tensor(legs, **dt)

    def gamma(self, q):
        M = torch.einsum("lk,lp,lq->kpq", self.pl, q, q)
        return quad_perm(M, self.w, self.tri, self.tri)

    def beta_norm2(self, q):
        B = torch.einsum("lk,el,lq->keq", self.pl, self.legs, q)
        K = torch.einsum("lk,el,fl->kef", self.pl, self.legs, self.legs)
        betas, n2s = [], []
        for e0, T in self.info:
            ri = torch.arange(e0, e0 + 3 * T, device=self.device).reshape(T, 3)
            betas.append(quad_perm(B, self.w, ri, self.tri).sum(0))
            n2s.append(quad_perm(K, self.w, ri, ri).sum())
        return torch.stack(betas), torch.stack(n2s)

    def alpha(self, q):
        beta, _ = self.beta_norm2(q)
        return torch.linalg.solve(self.gamma(q), beta.T).T

    def objective(self, q):
        G = self.gamma(q)
        beta, n2 = self.beta_norm2(q)
        alpha = torch.linalg.solve(G, beta.T).T
        return torch.mean((n2 - (beta * alpha).sum(1)) / n2)
