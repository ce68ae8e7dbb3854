"""FP64 NumPy oracle of the batched CF solver (test infrastructure only; the product never imports it).

Restates, for one instance of a batch made by sgl_analytic_gb300.cfbatch.make_batch:
  * the compensated per-plane sums Lambda_p(k) = sum_c w_c (e^{i k kap_c} - 1 - i k kap_c) (the kappa
    part of the reference's separable Psi_1, sgl_full.py:2596-2617);
  * gauss: ln Phi = sum_p Lambda_p - V k^2 / 2;
  * vp: ln Phi = sum_p Lambda_p + ln E exp(sum_p D_p(U_p) Lambda_p) over the stationary chain (weights w,
    transition K): the forward recursion alpha_1 = w e^{z_1}, alpha_{p+1} = (K^T alpha_p) e^{z_{p+1}}, as
    the reference's _chain_recursion (pos_closure.py:184-240) with one group per plane;
  * dP/dln mu = (1 - kappa) / 2 (1/pi) sum_n w_n Re[Phi(k_n) e^{-i k_n kappa}] on the uniform k grid with
    trapezoid weights, kappa = 1 - e^{-ln mu / 2}.
"""
from __future__ import annotations

import numpy as np


def plane_sums(batch, i):
    p0, p1, k = batch.instance(i)
    out = np.empty((p1 - p0, k.size), complex)
    for p in range(p0, p1):
        c0, c1 = batch.plane_cells[p], batch.plane_cells[p + 1]
        ph = np.outer(k, batch.kap[c0:c1])
        out[p - p0] = (np.expm1(1j * ph) - 1j * ph) @ batch.w[c0:c1]
    return out


def lnphi(batch, i):
    L = plane_sums(batch, i)
    p0, p1, k = batch.instance(i)
    if batch.closure[i] == 0:
        return L.sum(0) - 0.5 * batch.V[i] * k * k
    slot = int(np.sum(batch.closure[:i] == 1))
    K, w = batch.vp_K[slot], batch.vp_w[slot]
    D = batch.vp_D[p0:p1]
    lnsc = np.zeros(k.size)
    alpha = None
    for j in range(p1 - p0):
        z = D[j][:, None] * L[j][None, :]                     # (states, k)
        zmax = z.real.max(0)
        lnsc += zmax
        e = np.exp(z - zmax[None, :])
        alpha = (w[:, None] * e) if j == 0 else (K.T @ alpha) * e
        m = np.max(np.abs(alpha.real) + np.abs(alpha.imag), axis=0)
        alpha = alpha / m[None, :]
        lnsc += np.log(m)
    return L.sum(0) + lnsc + np.log(alpha.sum(0))


def pdf_lnmu(batch, i, lnmu, lnphi_i=None):
    p0, p1, k = batch.instance(i)
    L = lnphi(batch, i) if lnphi_i is None else lnphi_i
    return pdf_from_lnphi(L, k, lnmu)


def pdf_from_lnphi(L, k, lnmu):
    """dP/dln mu of the log-CF L on the uniform grid k (k[0] = 0)."""
    wk = np.full(k.size, k[1] - k[0])
    wk[0] *= 0.5
    wk[-1] *= 0.5
    cf = np.exp(L) * wk / np.pi
    kap = 1.0 - np.exp(-0.5 * np.asarray(lnmu, float))
    P = np.cos(np.outer(kap, k)) @ cf.real + np.sin(np.outer(kap, k)) @ cf.imag
    return P * (1.0 - kap) * 0.5
