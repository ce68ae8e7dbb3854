"""Batches of uneven instances for the batched CF solver (sgl_cfb_*).

An instance is a (cosmology, source redshift, closure) triple.  Its lens population is split into
planes z_l = z_s (j + 1/2) / n_p, j < n_p, with n_p rising from 32 at z_s = 0.3 to 256 at z_s = 5;
each plane holds the cells of the synthetic plane model (log-spaced halo masses x log-spaced
impact parameters, truncated-NFW convergence) scaled by the cosmology: the convergence by the
lensing efficiency D_l D_ls / D_s of a CPL (w0, wa) cosmology with curvature Ok, the rates by its
comoving volume per unit redshift and a mass cutoff set by sigma8.  Its k grid is uniform on
[0, k_max] with k_max = 40 / sigma_kappa (|Phi| ~ e^-800 there) and 4096 .. 32768 points.  Half the
instances use the gauss closure (a clustering variance V = 0.2 sigma_kappa^2), half the vp closure:
an 8-state stationary chain over the planes (Gauss-Hermite states, Gaussian-copula transitions with
line-of-sight correlation rho) with variance-preserving rectified rates per plane, the
one-dimensional form of the positive Cox closure (pos_closure.py:251-318; one group per plane).

The cosmology box and the sizes are those of the batched-solver benchmark: h, Om, sigma8, Ob, ns,
Ok, w0, wa in [0.6, 0.8] x [0.2, 0.4] x [0.7, 0.9] x [0.04, 0.06] x [0.92, 1.0] x [-0.05, 0.05] x
[-1.3, -0.7] x [-0.5, 0.5], z_s in [0.3, 5], Latin-hypercube seeded.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .workloads import nfw_trunc_projected

BOX = np.array([[0.6, 0.8], [0.2, 0.4], [0.7, 0.9], [0.04, 0.06], [0.92, 1.0], [-0.05, 0.05], [-1.3, -0.7],
                [-0.5, 0.5]])
ZS_RANGE = (0.3, 5.0)
NSTATE = 8


def latin_hypercube(n, d, rng):
    """n points in [0, 1)^d, one per stratum in every dimension."""
    u = (np.argsort(rng.random((d, n)), axis=1).T + rng.random((n, d))) / n
    return u


def planes_for(zs):
    return int(round(32 + 224 * (zs - ZS_RANGE[0]) / (ZS_RANGE[1] - ZS_RANGE[0])))


class PlaneCells:
    """Cells of one plane: nm log-spaced masses 1e8-1e16 Msun/h x nb log-spaced impact parameters
    1e-3-1e2 r_s; kappa = A(z_l) (M/1e12)^0.3 F(b; c(M)), c = 5 (M/1e12)^-0.1; rates
    w = R(z_l) M^-0.9 exp(-M/M*) dlnM 2 pi b^2 dlnb, M* = 1e15 (sigma8 / 0.811)^4."""

    def __init__(self, nm=16, nb=16):
        self.M = np.geomspace(1e8, 1e16, nm)
        self.b = np.geomspace(1e-3, 1e2, nb)
        c = 5.0 * (self.M / 1e12) ** -0.1
        F = nfw_trunc_projected(self.b[None, :], c[:, None])
        self.kapF = (((self.M / 1e12) ** 0.3)[:, None] * F).ravel()
        self.dlnM = math.log(self.M[1] / self.M[0])
        dlnb = math.log(self.b[1] / self.b[0])
        self.area = 2 * math.pi * self.b ** 2 * dlnb
        self.n_cells = nm * nb

    def weights(self, s8):
        Ms = 1e15 * (s8 / 0.811) ** 4
        nm = self.M ** -0.9 * np.exp(-self.M / Ms) * self.dlnM
        return (nm[:, None] * self.area[None, :]).ravel()


def comoving(theta, z):
    """Transverse comoving distance (units of c/H0) and E(z) at z for theta = (h, Om, s8, Ob, ns, Ok, w0, wa)."""
    h, Om, s8, Ob, ns, Ok, w0, wa = theta
    zz = np.linspace(0.0, float(np.max(z)), 4001)
    Ode = 1.0 - Om - Ok
    fde = (1 + zz) ** (3 * (1 + w0 + wa)) * np.exp(-3 * wa * zz / (1 + zz))
    E = np.sqrt(Om * (1 + zz) ** 3 + Ok * (1 + zz) ** 2 + Ode * fde)
    chi = np.concatenate([[0.0], np.cumsum(0.5 * (1 / E[1:] + 1 / E[:-1]) * np.diff(zz))])
    chi_z = np.interp(z, zz, chi)
    if Ok > 0:
        dm = np.sinh(math.sqrt(Ok) * chi_z) / math.sqrt(Ok)
    elif Ok < 0:
        dm = np.sin(math.sqrt(-Ok) * chi_z) / math.sqrt(-Ok)
    else:
        dm = chi_z
    return dm, np.interp(z, zz, E), chi_z


def plane_scales(theta, zs, zl):
    """(A, R) per plane: convergence scale (lensing efficiency) and rate scale (comoving volume)."""
    Ok = theta[5]
    z = np.concatenate([zl, [zs]])
    dm, E, chi = comoving(theta, z)
    Dl, Ds = dm[:-1], dm[-1]
    Dls = (Ds * np.sqrt(1 + Ok * Dl ** 2) - Dl * np.sqrt(1 + Ok * Ds ** 2))
    A = 0.6 * (Dl * Dls / Ds) * (theta[1] / 0.315) * (1 + zl)
    R = 2.0e7 * chi[:-1] ** 2 / E[:-1] * (theta[1] / 0.315) * (zs / len(zl))
    return A, R


def hermite_states(n=NSTATE):
    """Gauss-Hermite (probabilists') nodes and stationary weights summing to 1."""
    u, w = np.polynomial.hermite_e.hermegauss(n)
    return u, w / w.sum()


def copula_transition(u, w, rho, tol=3e-14):
    """Transition matrix K with stationary weights w from the Gaussian copula of correlation rho on
    the nodes u, balanced symmetrically until w is stationary (the construction of pos_closure.py's
    transition, restated)."""
    x, y = u[:, None], u[None, :]
    J = w[:, None] * w[None, :] * np.exp((2 * rho * x * y - rho * rho * (x * x + y * y)) / (2 * (1 - rho * rho)))
    v = np.ones(u.size)
    for _ in range(10000):
        marg = v * (J @ v)
        if np.max(np.abs(marg / w - 1)) < tol:
            break
        v *= np.sqrt(w / marg)
    return (v[:, None] * J * v[None, :]) / w[:, None]


def rectified_rates(var, u, w, iters=200):
    """Variance-preserving rectified rates lam(u) = (u - t)^+ / E_w[(u - t)^+] with E_w lam = 1 and
    Var_w lam = var per row of var (the vp rates of pos_closure.py:273-308, found here by bisection
    on the threshold t); below the first node's threshold the rate is the linear 1 + sqrt(var) u."""
    var = np.atleast_1d(np.asarray(var, float))
    lam = np.empty((var.size, u.size))

    def relvar(t):
        xx = np.maximum(u[None, :] - t[:, None], 0.0)
        e1 = xx @ w
        e2 = (xx * xx) @ w
        return e2 / e1 ** 2 - 1.0, xx, e1

    r0, _, _ = relvar(np.array([u[0]]))
    lin = var < r0[0]
    lam[lin] = 1.0 + np.sqrt(var[lin])[:, None] * u[None, :]
    idx = np.nonzero(~lin)[0]
    if idx.size:
        lo = np.full(idx.size, u[0])
        hi = np.full(idx.size, u[-2])
        for _ in range(iters):
            mid = 0.5 * (lo + hi)
            rv, _, _ = relvar(mid)
            up = rv < var[idx]
            lo = np.where(up, mid, lo)
            hi = np.where(up, hi, mid)
        _, xx, e1 = relvar(0.5 * (lo + hi))
        lam[idx] = xx / e1[:, None]
    return lam


@dataclass
class Batch:
    theta: np.ndarray          # (n, 8)
    zs: np.ndarray             # (n,)
    closure: np.ndarray        # (n,) 0 gauss, 1 vp
    inst_plane0: np.ndarray    # (n + 1,)
    plane_cells: np.ndarray    # (n_planes + 1,)
    kap: np.ndarray
    w: np.ndarray
    nk: np.ndarray
    dk: np.ndarray
    V: np.ndarray
    sigma: np.ndarray
    vp_D: np.ndarray           # (n_planes, NSTATE)
    vp_K: np.ndarray           # (n_vp, NSTATE, NSTATE)
    vp_w: np.ndarray           # (n_vp, NSTATE)
    nstate: int = NSTATE

    def arrays(self):
        return dict(inst_plane0=self.inst_plane0, plane_cells=self.plane_cells, kap=self.kap, w=self.w, nk=self.nk,
                    dk=self.dk, closure=self.closure, V=self.V, nstate=self.nstate, vp_D=self.vp_D, vp_K=self.vp_K,
                    vp_w=self.vp_w)

    @property
    def n_inst(self):
        return int(self.zs.size)

    def instance(self, i):
        """(planes' cell slices, k grid) of instance i (for oracles)."""
        p0, p1 = int(self.inst_plane0[i]), int(self.inst_plane0[i + 1])
        return p0, p1, np.arange(int(self.nk[i])) * float(self.dk[i])

    def terms(self):
        """(k-point, cell) terms of the whole batch."""
        cells = np.diff(self.plane_cells)
        per_inst = np.add.reduceat(cells, self.inst_plane0[:-1])
        return float(np.sum(per_inst.astype(float) * self.nk))


def make_batch(n_inst, seed=0, nm=16, nb=16, nk_range=(4096, 32768), nk_step=128, max_planes=None):
    """n_inst instances (Latin hypercube over BOX x z_s), alternating gauss / vp closures.
    max_planes caps the plane count (small test batches)."""
    rng = np.random.default_rng(seed)
    u = latin_hypercube(n_inst, 11, rng)
    theta = BOX[:, 0] + u[:, :8] * (BOX[:, 1] - BOX[:, 0])
    zs = ZS_RANGE[0] + u[:, 8] * (ZS_RANGE[1] - ZS_RANGE[0])
    nk = (nk_range[0] + np.floor(u[:, 9] * (nk_range[1] - nk_range[0]) / nk_step) * nk_step).astype(np.int32)
    rho = 0.3 + 0.5 * u[:, 10]
    closure = (np.arange(n_inst) % 2).astype(np.int32)
    pc = PlaneCells(nm, nb)
    us, ws = hermite_states()
    kap, w, p0, pcells, V, dk, sig, D, K, Wst = [], [], [0], [0], [], [], [], [], [], []
    for i in range(n_inst):
        npl = planes_for(zs[i]) if max_planes is None else min(planes_for(zs[i]), max_planes)
        zl = zs[i] * (np.arange(npl) + 0.5) / npl
        A, R = plane_scales(theta[i], zs[i], zl)
        wt = pc.weights(theta[i][2])
        kp = A[:, None] * pc.kapF[None, :]
        wp = R[:, None] * wt[None, :]
        kap.append(kp.ravel()); w.append(wp.ravel())
        pcells.extend((pcells[-1] + pc.n_cells * (np.arange(npl) + 1)).tolist())
        p0.append(p0[-1] + npl)
        s2 = float(np.sum(wp * kp * kp))
        sigma = math.sqrt(s2 * 1.2)                       # with the clustering part
        sig.append(sigma)
        V.append(0.2 * s2 if closure[i] == 0 else 0.0)
        dk.append(40.0 / sigma / (nk[i] - 1))
        if closure[i] == 1:
            # per-plane rate variance: 0.3 of the plane's share of the convergence variance, scaled to
            # the largest plane
            share = np.sum(wp * kp * kp, axis=1)
            D.append(rectified_rates(0.3 * share / share.max(), us, ws) - 1.0)
            K.append(copula_transition(us, ws, rho[i]))
            Wst.append(ws)
        else:
            D.append(np.zeros((npl, NSTATE)))
    return Batch(theta=theta, zs=zs, closure=closure, inst_plane0=np.array(p0, np.int32),
                 plane_cells=np.array(pcells, np.int64), kap=np.concatenate(kap), w=np.concatenate(w), nk=nk,
                 dk=np.array(dk), V=np.array(V), sigma=np.array(sig), vp_D=np.concatenate(D),
                 vp_K=np.array(K) if K else np.zeros((0, NSTATE, NSTATE)), vp_w=np.array(Wst) if Wst else np.zeros((0, NSTATE)))
