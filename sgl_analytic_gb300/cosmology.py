"""Cosmology tables on the GPU (sgl_cosmo_tables): the reference's chain Cosmology (sgl.py:65-640 as
pipeline.make_cosmology builds it, pipeline.py:39-79) for many cosmologies at once, and the lensing
critical surface density from its distances (Cosmology.Sigma_cr, sgl.py:240-255)."""
from __future__ import annotations

import numpy as np

CKMS = 299792.458            # km/s
GNEWT = 4.30091e-9           # Mpc (km/s)^2 / Msun
PARAM_KEYS = ("h", "Om", "Ob", "s8", "ns", "zeq", "Ok", "w0", "wa")
DEFAULT = dict(h=0.674, Om=0.315, Ob=0.0493, s8=0.811, ns=0.965, zeq=3402.0, Ok=0.0, w0=-1.0, wa=0.0)


def params_array(cosmologies):
    """(n, 9) rows from dicts (missing keys take the reference's defaults) or arrays."""
    rows = []
    for c in cosmologies:
        if isinstance(c, dict):
            unknown = set(c) - set(PARAM_KEYS)
            if unknown:
                raise ValueError(f"unknown cosmology parameter(s) {sorted(unknown)}")
            rows.append([float(c.get(k, DEFAULT[k])) for k in PARAM_KEYS])
        else:
            rows.append([float(v) for v in c])
    return np.array(rows)


def f_K(params_row, chi):
    """Transverse comoving distance of a radial interval chi [Mpc] (sgl.py:219-238)."""
    h, Ok = params_row[0], params_row[6]
    chi = np.asarray(chi, float)
    if Ok == 0.0:
        return chi
    u = chi * 100.0 * h / CKMS
    t = Ok * u * u
    x = np.sqrt(abs(Ok)) * u
    with np.errstate(invalid="ignore", divide="ignore"):
        ratio = np.sinh(x) / x if Ok > 0 else np.sin(x) / x
    ratio = np.where(abs(t) < 1e-5, 1 + t / 6 + t ** 2 / 120 + t ** 3 / 5040, ratio)
    return chi * ratio


def sigma_cr(engine, cosmologies, pairs):
    """Sigma_cr(z_l, z_s) [Msun / Mpc^2] of each cosmology at each (z_l, z_s) pair: (n, n_pairs)."""
    p = params_array(cosmologies)
    pairs = np.atleast_2d(np.asarray(pairs, float))
    z = np.unique(pairs.ravel())
    chi = engine.cosmo_tables(p, z, np.array([1e12]))["chi"]
    out = np.empty((p.shape[0], pairs.shape[0]))
    for i in range(p.shape[0]):
        c = dict(zip(z, chi[i]))
        for j, (zl, zs) in enumerate(pairs):
            DA_s = f_K(p[i], c[zs]) / (1 + zs)
            DA_l = f_K(p[i], c[zl]) / (1 + zl)
            DA_ls = f_K(p[i], c[zs] - c[zl]) / (1 + zs)
            out[i, j] = CKMS ** 2 * DA_s / (4 * np.pi * GNEWT * DA_l * DA_ls)
    return out
