"""FP64 CPU oracle for the Hankel/Fourier inversion ln Phi -> P_s(ln mu).

TEST INFRASTRUCTURE ONLY (the checker, never the product).  Restates, in NumPy/SciPy, the
reference package's (sgl_analytic v0.2.0) width-relative inversion:

* ``vector_grid``     <- ``sgl.vector_grid``          sgl.py:1229-1258, constants sgl.py:1176-1193
* ``reach``           <- ``sgl_full._reach``          sgl_full.py:38-47
* ``p_vector_joint``  <- ``sgl.P_vector_joint``       sgl.py:1127-1156
* ``plan_grid``       <- ``sgl_full.invert`` 187-262 (box, reach, k-steps, output grid)
* ``invert``          <- ``sgl_full.invert`` 159-375 (unblocked path, uniform output grid,
                         Euler-Maclaurin endpoint term, path integral, normalisation, moments)
"""
from __future__ import annotations

import numpy as np
import scipy.special as sp

# sgl.py:1176-1193
SIG_REACH = 12.0
PPP_K = 18.0
PPP_G = 96.0
BOX_REACH = 6.0
PTS_PER_SIG_KAP = 72.0
PTS_PER_SIG_GAM = 36.0
XI_REACH = 24.0
# sgl_full.py:33-36, 53-60
TAIL_KAP_MAX = 0.99
TAIL_GAM_MAX = 0.8
TAIL_PPP_G = 12.0
INVERT_BLOCK_PTS = 20_000_000
OUT_GRID_MAX = 3.4e7

trapz = np.trapezoid


def vector_grid(sigma, xi_reach=XI_REACH):
    """Width-relative grid (sgl.py:1229-1258)."""
    sig_xi = 2.0 * sigma
    xi_max = xi_reach * sig_xi
    xi_min = -BOX_REACH * sig_xi
    kap_max = 1.0 - np.exp(-0.5 * xi_max)
    kap_min = -BOX_REACH * sigma
    gam_max = BOX_REACH * sigma
    k_k_max = SIG_REACH / sigma
    k_g_max = SIG_REACH / sigma
    kap_ext = max(abs(kap_min), kap_max)
    dk_k = 2.0 * np.pi / (PPP_K * kap_ext)
    dk_g = 2.0 * np.pi / (PPP_G * gam_max)
    return dict(nk_k=int(np.ceil(k_k_max / dk_k)) + 1, nk_g=int(np.ceil(k_g_max / dk_g)) + 1,
                k_k_max=k_k_max, k_g_max=k_g_max,
                n_kap=int(np.ceil((kap_max - kap_min) / (sigma / PTS_PER_SIG_KAP))) + 1,
                n_gam=int(np.ceil(gam_max / (sigma / PTS_PER_SIG_GAM))) + 1,
                kap_min=kap_min, kap_max=kap_max, gam_max=gam_max,
                xi_min=xi_min, xi_max=xi_max, sigma=sigma)


def reach_points(k0, max_mult=64.0):
    """Probe points k0 * 1.25^j of _reach (sgl_full.py:40-41)."""
    mults = 1.25 ** np.arange(0, int(np.ceil(np.log(max_mult) / np.log(1.25))) + 1)
    return k0 * mults


def reach_pick(ks, L, tol):
    """First probe with |Phi| <= tol, else the smallest |Phi| (sgl_full.py:44-47)."""
    phi = np.abs(np.exp(L))
    ok = np.nonzero(phi <= tol)[0]
    i = int(ok[0]) if len(ok) else int(np.argmin(phi))
    return float(ks[i]), float(phi[i])


def reach(lam, k0, axis, tol):
    ks = reach_points(k0)
    zero = np.zeros(1)
    L = lam(ks, zero)[:, 0] if axis == "k" else lam(zero, ks)[0, :]
    return reach_pick(ks, L, tol)


def plan_grid(sigma, reach_fn, xi_reach=XI_REACH, tail_box=True, phi_tol=1e-8):
    """Grid selection of invert (sgl_full.py:187-262) for keep_dk=True, grid_scale=1, no
    override, no positive-closure coarse rule.  reach_fn(k0, axis) -> (k_max, |Phi| there).
    Returns the grid dict and the axes (k_k, k_g, kap, gam, g_def)."""
    grid = vector_grid(sigma, xi_reach=xi_reach)
    g0 = grid["gam_max"]
    kap_max = gam_max = None
    if tail_box:
        kap_max = max(grid["kap_max"], TAIL_KAP_MAX)
        gam_max = max(g0, TAIL_GAM_MAX)
    dk0 = (2 * np.pi / (PPP_K * max(abs(grid["kap_min"]), grid["kap_max"])),
           2 * np.pi / (PPP_G * grid["gam_max"]))
    if tail_box and gam_max is not None and TAIL_PPP_G:
        dk0 = (dk0[0], min(dk0[1], 2 * np.pi / (TAIL_PPP_G * gam_max)))
    if (kap_max is not None and kap_max != grid["kap_max"]) or \
            (gam_max is not None and gam_max != grid["gam_max"]):
        if kap_max is not None:
            grid["kap_max"] = float(kap_max)
        if gam_max is not None:
            grid["gam_max"] = float(gam_max)
        grid["n_kap"] = int(np.ceil((grid["kap_max"] - grid["kap_min"])
                                    / (sigma / PTS_PER_SIG_KAP))) + 1
        grid["n_gam"] = int(np.ceil(grid["gam_max"] / (sigma / PTS_PER_SIG_GAM))) + 1
    grid["k_k_max"], phi_k = reach_fn(grid["k_k_max"], "k")
    grid["k_g_max"], phi_g = reach_fn(grid["k_g_max"], "g")
    dk_k, dk_g = dk0
    grid["nk_k"] = int(np.ceil(grid["k_k_max"] / dk_k)) + 1
    grid["nk_g"] = int(np.ceil(grid["k_g_max"] / dk_g)) + 1
    grid.update(phi_at_k_cut=phi_k, phi_at_g_cut=phi_g)
    if grid["n_kap"] * grid["n_gam"] > OUT_GRID_MAX:
        raise NotImplementedError("geometric output grid (n_kap * n_gam > OUT_GRID_MAX)")
    k_k = np.linspace(0.0, grid["k_k_max"], grid["nk_k"])
    k_g = np.linspace(0.0, grid["k_g_max"], grid["nk_g"])
    kap = np.linspace(grid["kap_min"], grid["kap_max"], grid["n_kap"])
    gam = np.linspace(0.0, grid["gam_max"], grid["n_gam"])
    grid.update(window=0.0)
    return grid, k_k, k_g, kap, gam, min(g0, grid["gam_max"])


def p_vector_joint(k_k, k_g, Phi, kap, gam):
    """Hankel over k_gamma then Fourier over k_kappa (sgl.py:1127-1156)."""
    dk_k = k_k[1] - k_k[0]
    dk_g = k_g[1] - k_g[0]
    J0 = sp.j0(np.outer(gam, k_g))
    w_kg = np.full(k_g.size, dk_g)
    w_kg[0] *= 0.5
    w_kg[-1] *= 0.5
    F = Phi @ ((k_g * w_kg)[:, None] * J0.T)
    w_kk = np.full(k_k.size, dk_k)
    w_kk[0] *= 0.5
    w_kk[-1] *= 0.5
    E = np.exp(-1j * np.outer(kap, k_k))
    return (1.0 / (2.0 * np.pi ** 2)) * np.real(E @ (F * w_kk[:, None]))


def em_correction(k_k, k_g, Phi0, Phi1, kap, gam):
    """Euler-Maclaurin endpoint term of the k_gamma trapezoid (sgl_full.py:277-298):
    returns a(kap), b(kap) with P3 += a + b gam^2."""
    dkk, dkg = k_k[1] - k_k[0], k_g[1] - k_g[0]
    wkk = np.full(k_k.size, dkk)
    wkk[0] *= 0.5
    wkk[-1] *= 0.5
    Phi2 = (Phi1 - Phi0) / dkg ** 2
    c = 1.0 / (2.0 * np.pi ** 2)
    va = (dkg ** 2 / 12.0) * Phi0 - (dkg ** 4 / 120.0) * Phi2
    vb = (dkg ** 4 / 480.0) * Phi0
    E = np.exp(-1j * np.outer(kap, k_k)) * wkk[None, :]
    return c * np.real(E @ va), c * np.real(E @ vb)


def path_points(xi_grid, kap, gmax, g_def, dgam, n_k_int=2400):
    """All (kappa, gamma) points of the constant-mu paths of P_i (sgl_full.py:305-350).
    Returns (points (N, 2), segments [(i, kind, x, extra, pref, offset)])."""
    segs, pts = [], []
    off = 0
    for i, xi in enumerate(xi_grid):
        mu = np.exp(xi)
        rm = 1.0 / np.sqrt(mu)
        hi = 1.0 - rm
        lo = max(kap[0], 1.0 - np.sqrt(1.0 / mu + g_def ** 2))
        if hi <= lo:
            continue
        ke = np.linspace(lo, hi, n_k_int)
        ge = np.sqrt(np.clip((hi - ke) * (1.0 - ke + rm), 0.0, None))
        pts.append(np.column_stack([ke, ge]))
        segs.append((i, 0, ke, None, np.pi / mu ** 2, off))
        off += ke.size
        if gmax > g_def and lo > kap[0]:
            gb = min(gmax, np.sqrt(max((hi - kap[0]) * (1.0 - kap[0] + rm), 0.0)))
            if gb > g_def:
                n = int(np.ceil((gb - g_def) / (0.5 * dgam))) + 1
                gx = np.linspace(g_def, gb, n)
                r = np.sqrt(1.0 / mu + gx ** 2)
                kx = np.clip(1.0 - r, kap[0], kap[-1])
                pts.append(np.column_stack([kx, gx]))
                segs.append((i, 1, gx, gx / r, np.pi / mu ** 2, off))
                off += gx.size
    return (np.concatenate(pts) if pts else np.zeros((0, 2))), segs


def path_integral(P3, kap, gam, xi_grid, gmax, g_def, n_k_int=2400):
    """P_i (sgl_full.py:305-360): bilinear P3 along each constant-mu path, trapezoid."""
    from scipy.interpolate import RegularGridInterpolator
    ip = RegularGridInterpolator((kap, gam), P3, bounds_error=False, fill_value=0.0)
    out = np.zeros_like(xi_grid)
    pts, segs = path_points(xi_grid, kap, gmax, g_def, gam[1] - gam[0], n_k_int)
    if not segs:
        return out
    vals = ip(pts)
    for i, kind, xs, extra, pref, o in segs:
        v = vals[o:o + xs.size]
        if kind == 0:
            out[i] = pref * trapz(v, xs)
        else:
            out[i] += pref * trapz(v * extra, xs)
    return out


def finish(P3, kap, gam, grid, g_def, xi_out, n_xi_wide=500, n_k_int=2400):
    """Normalisation on the wide grid, moments, output (sgl_full.py:362-375)."""
    gmax = grid["gam_max"]
    xw = np.linspace(grid["xi_min"], grid["xi_max"], n_xi_wide)
    pw = path_integral(P3, kap, gam, xw, gmax, g_def, n_k_int)
    norm = trapz(pw, xw)
    ps = pw / norm
    mean = float(trapz(xw * ps, xw))
    var = float(trapz((xw - mean) ** 2 * ps, xw))
    skew = float(trapz((xw - mean) ** 3 * ps, xw) / var ** 1.5)
    x = np.exp(-0.5 * xw)
    md = float(trapz(x * ps, xw))
    sDL = float(np.sqrt(trapz((x - md) ** 2 * ps, xw)) / md)
    Ps = path_integral(P3, kap, gam, np.asarray(xi_out, float), gmax, g_def, n_k_int) / norm
    return Ps, dict(mean=mean, var=var, skew=skew, sigmaDL=sDL, norm=norm)


def invert(lam, sigma, xi_out, tail_box=True, phi_tol=1e-8, n_xi_wide=500, n_k_int=2400,
           return_phi=False):
    """sgl_full.invert for the default gauss chain (unblocked, window=False)."""
    grid, k_k, k_g, kap, gam, g_def = plan_grid(
        sigma, lambda k0, ax: reach(lam, k0, ax, phi_tol), tail_box=tail_box, phi_tol=phi_tol)
    if k_k.size * k_g.size > INVERT_BLOCK_PTS:
        raise NotImplementedError("blocked inversion")
    Phi = np.exp(lam(k_k, k_g))
    P3 = p_vector_joint(k_k, k_g, Phi, kap, gam)
    a, b = em_correction(k_k, k_g, Phi[:, 0], Phi[:, 1], kap, gam)
    P3 = P3 + a[:, None] + b[:, None] * gam[None, :] ** 2
    Ps, meta = finish(P3, kap, gam, grid, g_def, xi_out, n_xi_wide, n_k_int)
    meta.update(grid=grid, P3=P3, kap=kap, gam=gam)
    if return_phi:
        meta.update(Phi=Phi, k_k=k_k, k_g=k_g)
    return np.asarray(xi_out, float), Ps, meta
