"""FP64 CPU oracle for the positive (vp) Cox closure's ln R on a (k_kappa, k_gamma) grid.

TEST INFRASTRUCTURE ONLY (the checker, never the product).  Restates, vectorised in NumPy, the
reference package's (sgl_analytic v0.2.0) evaluation of

    ln R(k, q) = ln E_U exp( sum_s sum_g (lam_g(U_s) - 1) Y_g(k, q) ),
    Y_g = sum_{c in g} w_c (e_c(k) J_c(q) + J_c(q) - 1),  e = expm1(i k kappa), J = J0(q gamma)

* group sums and rate-interval form of (lam - 1)  <- _fused_groups   pos_closure_fused.py:51-105
  (the rates are affine in the state u on one contiguous interval: rate_intervals, :18-48)
* 48-state stationary chain, forward recursion with max scaling <- _chain_recursion pos_closure.py:184-240
* the closure's Psi_2 replacement q_xi = unwrap(ln R) - shear_var q^2 / 4  <- Closure.qxi :690-705
"""
from __future__ import annotations

import numpy as np
from scipy.special import j0


def rate_matrix(ga, gb, gc, glo, ghi, u):
    """(G, nstate) values of lam_g(u_j) - 1 from the rate-interval parameters."""
    ns = u.size
    j = np.arange(ns)[None, :]
    lin = gc[:, None] == 0.0
    left = ghi[:, None] == ns - 1
    anchor = np.where(left[:, 0], u[glo], u[ghi])[:, None]
    active = (j >= glo[:, None]) & (j <= ghi[:, None])
    clipped = gc[:, None] + np.where(active, (u[None, :] - anchor) * ga[:, None] + gb[:, None], 0.0)
    return np.where(lin, ga[:, None] * u[None, :] + gb[:, None], clipped)


def z_tables(d, kv, qv):
    """z[s, state, point] (points k-major: p = i_k * nq + i_q) for every shell of closure data d."""
    kv, qv = np.asarray(kv, float), np.asarray(qv, float)
    e = np.expm1(1j * np.outer(d["ku"], kv))                     # (U, nk)
    J = j0(np.outer(d["gu"], qv))                                 # (U, nq)
    u = d["u"]
    nsh = d["sh_g"].size - 1
    P = kv.size * qv.size
    z = np.zeros((nsh, u.size, P), complex)
    D = rate_matrix(d["ga"], d["gb"], d["gc"], d["glo"], d["ghi"], u)
    gstart = d["gstart"]
    for s in range(nsh):
        g0, g1 = int(d["sh_g"][s]), int(d["sh_g"][s + 1])
        c0, c1 = int(gstart[g0]), int(gstart[g1])
        cu, cw = d["cu"][c0:c1], d["cw"][c0:c1]
        F = cw[:, None, None] * (e[cu][:, :, None] * J[cu][:, None, :] + (J[cu] - 1.0)[:, None, :])
        F = F.reshape(c1 - c0, P)
        Y = np.add.reduceat(F, gstart[g0:g1] - c0, axis=0) if g1 > g0 else np.zeros((0, P))
        empty = np.diff(gstart[g0:g1 + 1]) == 0
        Y[empty] = 0.0
        z[s] = D[g0:g1].T @ Y
    return z


def chain_lnR(z, K, w):
    """ln E exp(sum_s z_s(U_s)) for the stationary chain, log-scaled forward pass."""
    nsh, ns, P = z.shape
    scale = np.zeros(P)
    a = None
    for s in range(nsh):
        b = np.broadcast_to(w[:, None], (ns, P)).astype(complex) if s == 0 else K[s - 1].T @ a
        mx = z[s].real.max(axis=0)
        a = b * np.exp(z[s] - mx[None, :])
        nrm = np.max(np.abs(a), axis=0)
        a = a / nrm[None, :]
        scale += mx + np.log(nrm)
    t = a.sum(axis=0)
    return scale + 0.5 * np.log(t.real ** 2 + t.imag ** 2) + 1j * np.arctan2(t.imag, t.real)


def lnR(d, kv, qv):
    z = z_tables(d, kv, qv)
    return chain_lnR(z, d["K"], d["w"]).reshape(len(kv), len(qv))


def qxi(d, kk, kg):
    """unwrap(ln R) - shear_var kg^2 / 4 on the tensor grid (Closure.qxi, pos_closure.py:690-705)."""
    v = lnR(d, kk, kg)
    im = v.imag.copy()
    im[:, 0] = np.unwrap(im[:, 0])
    im = np.unwrap(im, axis=1)
    return v.real + 1j * im - 0.25 * float(d["shear_var"]) * np.asarray(kg, float)[None, :] ** 2
