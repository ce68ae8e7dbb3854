"""FP64 NumPy oracle of the surrogate + judge assembly (test infrastructure only; the product never
imports it).

Restates, for the tables of sgl_analytic_gb300.surrogate.SweepTables and the ensemble's normalised node
outputs Y[member][plane * nq + j] = (y0, y1):
  * the residual at ln q: r = (y0 scale + shift, y1 scale), 4-point Lagrange interpolation on the
    plane's nodes ln q_j = lnq0 + j hq (stencil j - 1 .. j + 2, j clamped to 1 .. nq - 3), and
    r(q0) q / q0 below the first node;
  * H = -exp(r0 + ln(mu2 / 2) + 2 ln q - ln(1 + (q Sbar)^2) / 2 + i (r1 + atan(q Sbar))), Sbar =
    mu2 / (2 mu1), per member; the mean over members and the spread 2 max_m |H_m - mean|;
  * ln Phi(k_n) = sum_p dz_p mean_p(s_p k_n), n >= 1 (0 at k = 0), per instance;
  * the judge's per-plane maxima of dz spread (as is, and times |Phi| of the surrogate sum) and the k
    band [first n, 1 + last n] whose weighted spread exceeds tau ((0, 0) if none).
"""
from __future__ import annotations

import numpy as np


def _residual(Yp, x, dl, nq, scale, shift):
    below = x < 0
    j = np.clip(np.floor(x).astype(np.int64), 1, nq - 3)
    u = x - j
    um, u1, u2 = u + 1, u - 1, u - 2
    w = np.stack([-u * u1 * u2 / 6, um * u1 * u2 / 2, -um * u * u2 / 2, um * u * u1 / 6])
    idx = j[None, :] + np.arange(-1, 3)[:, None]
    r = np.stack([np.sum(w * Yp[idx, c], 0) for c in (0, 1)], -1)
    r0 = np.stack([np.full(x.size, Yp[0, 0]), np.full(x.size, Yp[0, 1])], -1)
    r = np.where(below[:, None], r0 * np.exp(np.minimum(dl, 0))[:, None], r)
    return np.stack([r[:, 0] * scale + shift, r[:, 1] * scale], -1)


def plane_H(tables, Y, p, k, shift, scale):
    """(members, k) H of plane p at k > 0."""
    nq = tables.nq
    lq = np.log(tables.s[p] * k)
    x = (lq - tables.lnq0[p]) / tables.hq[p]
    dl = lq - tables.lnq0[p]
    qs = np.exp(lq) * tables.mu2[p] / (2 * tables.mu1[p])
    b0 = np.log(0.5 * tables.mu2[p]) + 2 * lq - 0.5 * np.log1p(qs * qs)
    b1 = np.arctan(qs)
    out = []
    for m in range(Y.shape[0]):
        Yp = Y[m, p * nq:(p + 1) * nq].astype(np.float64)
        r = _residual(Yp, x, dl, nq, scale, shift)
        out.append(-np.exp(r[:, 0] + b0 + 1j * (r[:, 1] + b1)))
    return np.array(out)


def assemble(tables, Y, shift, scale, tau=0.0):
    """(ln Phi per instance (list of arrays), dis (planes, 2), band (planes, 2))."""
    lnphi, dis, band = [], np.zeros((tables.n_planes, 2)), np.zeros((tables.n_planes, 2), np.int64)
    for i in range(tables.zs.size):
        k = np.arange(int(tables.nk[i])) * tables.dk[i]
        p0, p1 = int(tables.inst_plane0[i]), int(tables.inst_plane0[i + 1])
        L = np.zeros(k.size, complex)
        spreads = []
        for p in range(p0, p1):
            H = plane_H(tables, Y, p, k[1:], shift, scale)
            mean = H.mean(0)
            spreads.append(2 * np.max(np.abs(H - mean[None, :]), 0) * tables.dz[p])
            L[1:] += tables.dz[p] * mean
        lnphi.append(L)
        phim = np.exp(L.real[1:])
        for p, sp in zip(range(p0, p1), spreads):
            dis[p] = (sp.max(), (sp * phim).max())
            above = np.nonzero(sp * phim > tau)[0]
            if above.size:
                band[p] = (above[0] + 1, above[-1] + 2)
    return lnphi, dis, band
