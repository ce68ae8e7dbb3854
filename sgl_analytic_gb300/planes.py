"""Synthetic lens planes of the per-plane log-CF surrogate and of its production sweep.

A plane at redshift z_l of a cosmology theta = (h, Om, sigma8, Ok, w0, wa) holds NM x NB cells: NM
log-spaced halo masses 1e8-1e16 Msun/h x NB log-spaced impact parameters 1e-3-1e2 r_s (the shapes of
the CF-sweep microbenchmark).  In source-independent units a cell has the surface density

    S_mb = (h / 0.674) (M / 1e12)^(0.3 + 0.1 ln(1 + z_l)) F(b; c(M)),   c = 5 (M / 1e12)^-0.1,

F the projected truncated-NFW shape, and the rate per unit redshift

    w_mb = C_R chi(z_l)^2 / E(z_l) (Om / 0.315) D(z_l)^4 M^-0.9 exp(-M / M*) dlnM 2 pi b^2 dlnb,
    M* = 1e15 (sigma8 D(z_l) / 0.811)^4,

with D the linear growth factor (growth index gamma = 0.55 + 0.05 (1 + w(z)), Linder 2005, Phys. Rev. D
72, 043529) and chi, E the comoving distance and expansion rate of CPL dark energy (w = w0 + wa z / (1 + z))
with curvature Ok, distances in c / H0.  For a source at z_s the convergence is kappa = s S with the
lensing efficiency s = 1.5 Om (1 + z_l) D_l D_ls / D_s (transverse comoving distances).  A plane of
thickness dz adds Lambda_p(k) = dz H(s k) to the source's log-CF, with the source-independent

    H(q; theta, z_l) = sum_mb w_mb (e^{i q S_mb} - 1 - i q S_mb),

the function the surrogate learns.  C_R is fixed so that the fiducial cosmology's z_s = 1 convergence
has sigma_kappa = 0.036 (the width of the reference's z_s = 1 population); sigma_kappa then runs from
0.011 at z_s = 0.5 to 0.20 at z_s = 10.

An instance (theta, z_s) has n_p = clip(round(64 z_s^0.6), 16, 256) planes at z_l = z_s (j + 1/2) / n_p
with dz = z_s / n_p, and a uniform k grid k_n = n dk, n < nk, reaching k_max = 30 / sigma_kappa.
"""
from __future__ import annotations

import math

import numpy as np

from .workloads import nfw_trunc_projected

NM, NB = 256, 512
BOX = np.array([[0.6, 0.8], [0.2, 0.4], [0.7, 0.9], [-0.05, 0.05], [-1.3, -0.7], [-0.5, 0.5]])
FIDUCIAL = np.array([0.674, 0.315, 0.811, 0.0, -1.0, 0.0])
ZMAX = 10.0
ZS_RANGE = (0.1, 10.0)
SIGMA_FID = 0.036
KFAC = 30.0
_NZ = 2001


def n_planes(zs):
    return int(np.clip(round(64.0 * float(zs) ** 0.6), 16, 256))


class Background:
    """Distances, expansion rate and growth of many cosmologies on one z grid [0, ZMAX]: arrays
    (n_theta, _NZ)."""

    def __init__(self, theta):
        th = np.atleast_2d(np.asarray(theta, float))
        self.theta = th
        h, Om, s8, Ok, w0, wa = (th[:, i:i + 1] for i in range(6))
        z = np.linspace(0.0, ZMAX, _NZ)[None, :]
        self.z = z[0]
        Ode = 1.0 - Om - Ok
        fde = (1 + z) ** (3 * (1 + w0 + wa)) * np.exp(-3 * wa * z / (1 + z))
        E2 = Om * (1 + z) ** 3 + Ok * (1 + z) ** 2 + Ode * fde
        E = np.sqrt(E2)
        dz = self.z[1] - self.z[0]
        inv = 1.0 / E
        chi = np.concatenate([np.zeros((th.shape[0], 1)), np.cumsum(0.5 * (inv[:, 1:] + inv[:, :-1]) * dz, 1)], 1)
        Omz = Om * (1 + z) ** 3 / E2
        gam = 0.55 + 0.05 * (1 + w0 + wa * z / (1 + z))
        f = Omz ** gam / (1 + z)
        lnD = -np.concatenate([np.zeros((th.shape[0], 1)), np.cumsum(0.5 * (f[:, 1:] + f[:, :-1]) * dz, 1)], 1)
        self.E, self.chi, self.D = E, chi, np.exp(lnD)
        sk = np.sqrt(np.abs(Ok))
        with np.errstate(invalid="ignore", divide="ignore"):
            dm_pos = np.sinh(sk * chi) / np.where(sk > 0, sk, 1.0)
            dm_neg = np.sin(sk * chi) / np.where(sk > 0, sk, 1.0)
        self.DM = np.where(Ok > 0, dm_pos, np.where(Ok < 0, dm_neg, chi))
        self.Ok = Ok[:, 0]

    def at(self, name, i, z):
        """Linear interpolation of table `name` of cosmology i at redshifts z."""
        return np.interp(z, self.z, getattr(self, name)[i])


class PlaneModel:
    """The cells of planes, their analytic second moment, and the instances' lensing efficiencies."""

    def __init__(self):
        self.M = np.geomspace(1e8, 1e16, NM)
        self.b = np.geomspace(1e-3, 1e2, NB)
        c = 5.0 * (self.M / 1e12) ** -0.1
        self.F = nfw_trunc_projected(self.b[None, :], c[:, None])                # (NM, NB)
        self.lnMr = np.log(self.M / 1e12)
        self.dlnM = math.log(self.M[1] / self.M[0])
        dlnb = math.log(self.b[1] / self.b[0])
        self.area = 2 * math.pi * self.b ** 2 * dlnb
        self.G1 = self.F @ self.area                                               # sum_b area F, per mass
        self.G2 = (self.F ** 2) @ self.area                                        # sum_b area F^2, per mass
        self.C_R = 1.0
        s2 = self.sigma2(FIDUCIAL, 1.0)
        self.C_R = SIGMA_FID ** 2 / s2

    # -------------------------------------------------------------- per plane (source-independent)
    def _plane_params(self, bg, i, zl):
        th = bg.theta[i]
        zl = np.atleast_1d(np.asarray(zl, float))
        chi, E, D = bg.at("chi", i, zl), bg.at("E", i, zl), bg.at("D", i, zl)
        alpha = 0.3 + 0.1 * np.log1p(zl)
        s_amp = th[0] / 0.674
        w_amp = self.C_R * chi ** 2 / E * (th[1] / 0.315) * D ** 4
        Ms = 1e15 * (th[2] * D / 0.811) ** 4
        return alpha, s_amp, w_amp, Ms

    def factors(self, bg, i, zl):
        """Per-mass factors (a, c), (len(zl), NM): the planes' cells are S = a[m] F[m, b], w = c[m] area[b]."""
        alpha, s_amp, w_amp, Ms = self._plane_params(bg, i, zl)
        a = s_amp * np.exp(alpha[:, None] * self.lnMr[None, :])
        c = w_amp[:, None] * (self.M[None, :] ** -0.9 * np.exp(-self.M[None, :] / Ms[:, None]) * self.dlnM)
        return a, c

    def cells(self, bg, i, zl):
        """(S, w) of the plane at zl of cosmology i of `bg`, flattened (NM * NB)."""
        a, c = self.factors(bg, i, np.array([float(zl)]))
        return (a[0][:, None] * self.F).ravel(), (c[0][:, None] * self.area[None, :]).ravel()

    def moments(self, bg, i, zl):
        """(mu1, mu2) = (sum_mb w S, sum_mb w S^2) of the planes at zl (the cells' sums in closed form)."""
        alpha, s_amp, w_amp, Ms = self._plane_params(bg, i, zl)
        nm = self.M[None, :] ** -0.9 * np.exp(-self.M[None, :] / Ms[:, None]) * self.dlnM
        e = np.exp(alpha[:, None] * self.lnMr[None, :])
        return w_amp * s_amp * ((nm * e) @ self.G1), w_amp * s_amp ** 2 * ((nm * e * e) @ self.G2)

    def mu2(self, bg, i, zl):
        return self.moments(bg, i, zl)[1]

    # -------------------------------------------------------------- instances
    @staticmethod
    def efficiency(bg, i, zs, zl):
        """Lensing efficiency s = 1.5 Om (1 + z_l) D_l D_ls / D_s of planes zl for a source at zs."""
        Ok = bg.Ok[i]
        Dl, Ds = bg.at("DM", i, zl), float(bg.at("DM", i, zs))
        Dls = Ds * np.sqrt(1 + Ok * Dl ** 2) - Dl * math.sqrt(1 + Ok * Ds ** 2)
        return 1.5 * bg.theta[i, 1] * (1 + zl) * Dl * np.maximum(Dls, 0.0) / Ds

    def instance(self, bg, i, zs):
        """Planes (zl, dz, s) and the analytic sigma_kappa of the source at zs for cosmology i."""
        n = n_planes(zs)
        zl = zs * (np.arange(n) + 0.5) / n
        dz = np.full(n, zs / n)
        s = self.efficiency(bg, i, zs, zl)
        sig2 = float(np.sum(dz * s ** 2 * self.mu2(bg, i, zl)))
        return zl, dz, s, math.sqrt(sig2)

    def sigma2(self, theta, zs):
        bg = Background(theta)
        return self.instance(bg, 0, zs)[3] ** 2


def k_grid(sigma, nk):
    """(dk, k) of an instance: uniform, k_max = KFAC / sigma_kappa."""
    dk = KFAC / sigma / (nk - 1)
    return dk, np.arange(nk) * dk
