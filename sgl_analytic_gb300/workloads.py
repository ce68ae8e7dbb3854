"""Workloads with the reference's z_s=1 shapes, built from committed data.

``zs1_population()``: the reference's own z_s=1 default-cosmology population -- all 79,574
occupied fine cells (tests/golden/pop_zs1_sub.npz) -- with 201 xi_lin groups (67 shells x
m = 0, 1, 2, as the reference's z_s=1 build has).  The full groups are 290 MB and are not
committed; each shell's groups are synthesised from the three real groups of shell 30 (their
coarse-cell patterns and rows), scaled to that shell's real Frobenius row norm
(tests/golden/zs1_xi_shell_stats.npz).  Shapes, sizes and cost per PDF are those of the real
problem; the xi values are a deterministic stand-in.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .population import Population

GOLDEN = Path(__file__).resolve().parents[1] / "tests" / "golden"
BASE_SHELL = 30


def zs1_population(golden: Path = GOLDEN) -> Population:
    pop = Population.load(golden / "pop_zs1_sub.npz")
    st = np.load(golden / "zs1_xi_shell_stats.npz")
    norms = st["norms"]
    base = pop.groups()
    m, nrow, nidx, idx, rows = [], [], [], [], []
    for s in range(norms.shape[0]):
        for g in base:
            f = norms[s, g["m"]] / norms[BASE_SHELL, g["m"]]
            m.append(g["m"])
            nrow.append(g["rows"].shape[0])
            nidx.append(g["idx"].size)
            idx.append(g["idx"])
            rows.append((g["rows"] * f).ravel())
    pop.xg_m = np.asarray(m, np.int32)
    pop.xg_nrow = np.asarray(nrow, np.int32)
    pop.xg_nidx = np.asarray(nidx, np.int32)
    pop.xg_idx = np.concatenate(idx).astype(np.int32)
    pop.xg_rows = np.concatenate(rows)
    pop.xg_s0 = float(st["s0"])
    return pop


def nfw_trunc_projected(x, c):
    """Projected density shape F(x; c) of an NFW profile truncated at r = c r_s (Takada & Jain 2003,
    MNRAS 340, 580, their eq. 27): Sigma(x) = 2 rho_s r_s F(x), x = R / r_s; zero beyond x = c."""
    x, c = np.broadcast_arrays(np.asarray(x, float), np.asarray(c, float))
    out = np.zeros_like(x)
    inside = x < c
    a = np.sqrt(np.maximum(c ** 2 - x ** 2, 0.0))
    arg = (x ** 2 + c) / (x * (1.0 + c))
    lo = inside & (x < 1.0 - 1e-6)
    hi = inside & (x > 1.0 + 1e-6)
    mid = inside & ~lo & ~hi
    out[lo] = (-a[lo] / ((1 - x[lo] ** 2) * (1 + c[lo]))
               + np.arccosh(arg[lo]) / (1 - x[lo] ** 2) ** 1.5)
    out[hi] = (-a[hi] / ((1 - x[hi] ** 2) * (1 + c[hi]))
               - np.arccos(np.clip(arg[hi], -1.0, 1.0)) / (x[hi] ** 2 - 1) ** 1.5)
    out[mid] = np.sqrt(c[mid] ** 2 - 1) / (3 * (1 + c[mid])) * (1 + 1 / (c[mid] + 1))
    return out


def cf_sweep_problem(seed=0, nz=128, nm=256, nb=512, nk=16384, total_rate=3.7e6):
    """The synthetic plane x mass x impact-parameter CF sweep (nz * nm * nb cells, nk k-points).

    Lens planes z in (0, 1) for a source at z_s = 1; masses log-spaced 1e8-1e16 Msun/h;
    impact parameters log-spaced 1e-3-1e2 r_s; concentration c = 5 (M / 1e12)^-0.1;
    kappa = kappa_s(M, z) F(b; c) with kappa_s = 0.05 (M / 1e12)^0.3 * 4 z (1 - z) (a lensing
    efficiency shaped amplitude); rates proportional to M^-0.9 exp(-M / 1e15) x Gaussian(z; 0.5, 0.3)
    x 2 pi b db x dlnM x dz, with a seeded lognormal (sigma 0.1) jitter per (z, M), normalised to a
    total expected count of total_rate; k log-spaced in [1e-2, 1e6].  Returns (kap, w, kk)."""
    rng = np.random.default_rng(seed)
    z = np.linspace(0.02, 0.98, nz)
    M = np.geomspace(1e8, 1e16, nm)
    b = np.geomspace(1e-3, 1e2, nb)
    dlnb = np.log(b[1] / b[0])
    dlnM = np.log(M[1] / M[0])
    dz = z[1] - z[0]
    c = 5.0 * (M / 1e12) ** -0.1
    F = nfw_trunc_projected(b[None, :], c[:, None])                        # (nm, nb)
    ks = 0.05 * (M / 1e12) ** 0.3                                           # (nm,)
    eff = 4.0 * z * (1.0 - z)                                               # (nz,)
    kap = eff[:, None, None] * ks[None, :, None] * F[None, :, :]            # (nz, nm, nb)
    dn = M ** -0.9 * np.exp(-M / 1e15) * dlnM                               # (nm,)
    gz = np.exp(-0.5 * ((z - 0.5) / 0.3) ** 2) * dz                         # (nz,)
    jit = np.exp(0.1 * rng.standard_normal((nz, nm)))
    area = 2 * np.pi * b * b * dlnb                                         # 2 pi b db with db = b dlnb
    w = (gz[:, None] * dn[None, :] * jit)[:, :, None] * area[None, None, :]
    w *= total_rate / w.sum()
    kk = np.geomspace(1e-2, 1e6, nk)
    return kap.ravel(), w.ravel(), kk


def deposit_node(seed=0, n_host=2048, n_fil=512, nphi=12, nx=260, nu=120):
    """One lens-redshift node's deposits, shaped like the population build's emitters (sgl_full.py:1848-2011):
    n_host pseudo-elliptical truncated NFW hosts, each nphi orientations x nx radial cells (kappa from the
    truncated projected profile times 1 + eps cos 2 phi, gamma 0.8 kappa, weights N_bar d(x^2) / x_m^2 / nphi,
    lens distance R = x r_s), and n_fil filaments of nu cells x nphi orientations (kappa of a cylinder core,
    gamma kappa / 2, untangential).  Masses log-uniform, kappa_s over 1e-4..3, seeded.  Returns a list of
    objects for Cells.add_many (with R and tang) and the node's dchi."""
    rng = np.random.default_rng(seed)
    phis = (np.arange(nphi) + 0.5) * (0.5 * np.pi / nphi)
    objs = []
    for h in range(n_host):
        ks = float(np.exp(rng.uniform(np.log(1e-4), np.log(3.0))))
        c = float(rng.uniform(3.0, 12.0))
        rs = float(np.exp(rng.uniform(np.log(0.02), np.log(0.4))))
        eps = float(rng.uniform(0.0, 0.3))
        nbar = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e3))))
        xm = c * 1.5
        xe = np.concatenate([[0.0], xm * np.geomspace(1e-6, 1.0, nx)])
        xc = np.where(xe[:-1] > 0, np.sqrt(xe[:-1] * np.maximum(xe[1:], 1e-300)), 0.5 * xe[1])
        base = ks * 4.0 * nfw_trunc_projected(xc, c)
        K = (base[None, :] * (1.0 + eps * np.cos(2 * phis)[:, None])).ravel()
        G = 0.8 * K
        W = np.tile(nbar * (xe[1:] ** 2 - xe[:-1] ** 2) / xm ** 2 / nphi, nphi)
        objs.append(dict(K=K, G=G, W=W, R=np.tile(xc * rs, nphi), shell=0, beta=float(rng.uniform(0.8, 3.0)),
                         tang=True))
    for f in range(n_fil):
        k0 = float(np.exp(rng.uniform(np.log(1e-4), np.log(0.3))))
        rsf = float(np.exp(rng.uniform(np.log(0.05), np.log(2.0))))
        ue = np.concatenate([[0.0], np.geomspace(1e-5, 1.0, nu)])
        uc = np.where(ue[:-1] > 0, np.sqrt(ue[:-1] * np.maximum(ue[1:], 1e-300)), 0.5 * ue[1])
        kk = k0 * np.sqrt(np.maximum(1.0 - uc ** 2, 0.0))
        K = np.repeat(kk[:, None], nphi, 1).ravel() * np.tile(1.0 / np.maximum(np.cos(phis), 0.1), nu) / 10.0
        W = np.repeat(((ue[1:] ** 2 - ue[:-1] ** 2))[:, None], nphi, 1).ravel() * float(rng.uniform(0.1, 10.0)) / nphi
        objs.append(dict(K=K, G=0.5 * K, W=W, R=np.repeat(uc * rsf, nphi), shell=0,
                         beta=float(rng.uniform(0.5, 2.0)), tang=False))
    return objs, 40.0
