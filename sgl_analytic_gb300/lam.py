"""Drop-in ``Lam`` and ``invert`` for the reference's hot path, evaluated on the GPU.

``Lam(cells, ...)`` takes the same arguments as the reference's ``sgl_full.Lam``
(sgl_full.py:2728-2733) and exposes the same call surface used by ``invert`` and ``pipeline.run``:
``lam(kk, kg)`` -> complex ln Phi on the tensor grid, ``lam.sigma()``.  ``invert(lam, sigma, ...)``
takes the reference's ``sgl_full.invert`` arguments (sgl_full.py:159-162) and returns
``(xi_out, P_s, meta)``.

Only the default chain is implemented (C=None, nord=1, no exact-S, lss_var=0, lam_coarse=0,
gauss xi_lin or vp closure, keep_dk, Euler-Maclaurin term, uniform output grid, unblocked
inversion); anything else raises NotImplementedError -- there is no CPU fallback.

The vp closure (``Lam.install_vp``) takes the arrays the reference's ``pos_closure.install``
(pos_closure.py:708-733) builds -- the 48-state chain, the per-shell groups and FusedVP's rate
intervals -- and routes the xi term through the GPU's ln R, as the reference routes ``Lam._Qxi``.
"""
from __future__ import annotations

import numpy as np

from ._lib import PRECISIONS, Engine
from .population import Population

PHI_TOL = 1e-10      # sgl.py:1178 (reference default of invert's phi_tol)
XI_REACH = 24.0      # sgl.py:1186


def _precision(p):
    if isinstance(p, str):
        if p not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, got {p!r}")
        return PRECISIONS[p]
    return int(p)


class Lam:
    """ln Phi(k_kappa, k_gamma) of a built population, on the GPU (reference: sgl_full.Lam)."""

    def __init__(self, cells, C=None, nord=None, chunk=8, k3=True, exactS=False, nsamp=2_000_000, seed=0,
                 centroid=True, s_taper="cos2", s_is=True, is_alpha=0.5, is_levels=(0.1, 0.4, 1.0),
                 q_coarse=101, lss_var=0.0, lam_coarse=0, lam_method="sep", xi=False, xi_coarse=101,
                 xi_prune=1e-7, xi_clamp=False, precision="fp64", device=0, engine=None):
        if C is not None:
            raise NotImplementedError("Cox shell covariance C (clustering != 'xilin') is not on the GPU path")
        if exactS:
            raise NotImplementedError("exact-S correction is not on the GPU path")
        if lss_var:
            raise NotImplementedError("lss_var (clustering='limber') is not on the GPU path")
        if lam_coarse:
            raise NotImplementedError("lam_coarse is not on the GPU path")
        if xi_clamp:
            raise NotImplementedError("xi_clamp is not on the GPU path")
        if xi and xi_coarse != 101:
            raise NotImplementedError("only xi_coarse=101 is implemented")
        if not centroid:
            raise NotImplementedError("centroid=False is not on the GPU path")
        if s_taper not in ("cos2", "linear"):
            raise ValueError("s_taper must be 'cos2' or 'linear'")
        if lam_method not in ("sep", "direct"):
            raise ValueError(f"lam_method must be 'sep' or 'direct', got {lam_method!r}")
        pop = cells if isinstance(cells, Population) else Population.from_cells(cells)
        if xi and not pop.has_xi:
            raise ValueError("Lam(xi=True) needs a population built with xi=")
        self.population = pop
        self.precision = _precision(precision)
        self.engine = engine if engine is not None else Engine(device)
        self.engine.set_cells(pop.w0, pop.k0, pop.g0, pop.ig, pop.fe_g, pop.V)
        self.xi_on = bool(xi)
        if self.xi_on:
            self.engine.set_xi(pop.xg_m, pop.xg_nrow, pop.xg_nidx, pop.xg_idx, pop.xg_rows, pop.ce_k, pop.ce_g,
                               prune=xi_prune or 0.0, s0=pop.xg_s0)
        else:
            self.engine.set_xi(np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32),
                               np.zeros(0, np.int32), np.zeros(0), np.array([-1.0, 1.0]), np.array([1e-9, 1.0]))
        self.xi_coarse = int(xi_coarse) if xi else 0
        self.V = float(pop.V)
        self.nord, self.k3, self.exactS, self.s_taper, self.C = 1, False, False, s_taper, None
        self.lam_coarse = 0
        self.lss_var = 0.0
        self.pos = None
        self.xi_coarse_rule = False

    VP_KEYS = ("u", "w", "K", "ku", "gu", "cu", "cw", "gstart", "sh_g", "ga", "gb", "gc", "glo", "ghi", "shear_var")

    def install_vp(self, closure):
        """Routes the xi term through the positive (vp) closure (pos_closure.install, kind="vp").

        closure: a mapping with the arrays of ``VP_KEYS`` (u, w: the 48 state nodes and stationary
        weights; K: (shells - 1, 48, 48) transition matrices; ku, gu: unique cell kappa / gamma; cu,
        cw: group members and weights; gstart, sh_g: group and shell offsets; ga, gb, gc, glo, ghi:
        FusedVP's rate intervals; shear_var).  None removes the closure."""
        if closure is None:
            self.engine.set_vp(None)
            self.pos, self.xi_coarse_rule = None, False
            return None
        if not self.xi_on:
            raise ValueError("the vp closure replaces the xi term: build Lam with xi=True")
        missing = [k for k in self.VP_KEYS if k not in closure]
        if missing:
            raise ValueError(f"vp closure is missing {missing}")
        self.engine.set_vp({k: closure[k] for k in self.VP_KEYS})
        self.pos = {k: closure[k] for k in self.VP_KEYS}
        self.xi_coarse_rule = True
        return self.pos

    def lnR(self, kv, qv, precision=None):
        """ln R of the installed vp closure on kv x qv (FusedVP.lnR_blocked, principal branch)."""
        p = self.precision if precision is None else _precision(precision)
        return self.engine.vp_lnR(np.asarray(kv, float), np.asarray(qv, float), p)

    def __call__(self, kk, kg, nproc=1):
        return self.engine.lnphi(np.asarray(kk, float), np.asarray(kg, float), self.precision)

    def sigma(self):
        return self.engine.sigma()


def invert(lam, sigma, xi_out=None, n_k_int=2400, xi_reach=XI_REACH, n_xi_wide=500, grid_scale=1.0,
           kap_max=None, gam_max=None, keep_dk=True, hankel_em=True, tail_box=True, phi_tol=PHI_TOL, nproc=1,
           window=False, precision=None, **override):
    """Phi = exp(lam) -> P_s(ln mu) on the GPU (reference: sgl_full.invert, sgl_full.py:159-375)."""
    if not isinstance(lam, Lam):
        raise TypeError("invert needs a sgl_analytic_gb300.Lam (the inversion runs on the GPU)")
    if grid_scale != 1.0 or kap_max is not None or gam_max is not None or not keep_dk or not hankel_em \
            or override:
        raise NotImplementedError("only the default inversion grid (keep_dk, Euler-Maclaurin, no overrides) "
                                  "is on the GPU path")
    if window not in (False, None, True, "auto"):
        raise ValueError(f"window must be True, False or 'auto', got {window!r}")
    if xi_out is None:
        xi_out = np.linspace(-0.35, 0.55, 160)
    xi_out = np.asarray(xi_out, float)
    sig = lam.sigma()
    if not np.isclose(sig, float(sigma), rtol=1e-12, atol=0.0):
        raise NotImplementedError("invert(sigma=...) must be lam.sigma() on the GPU path")
    p = lam.precision if precision is None else _precision(precision)
    Ps, m = lam.engine.pdf(xi_out, precision=p, tail_box=tail_box, phi_tol=phi_tol, n_xi_wide=n_xi_wide,
                           n_k_int=n_k_int, xi_reach=xi_reach, window=window)
    grid = dict(nk_k=int(m["nk_k"]), nk_g=int(m["nk_g"]), k_k_max=m["k_k_max"], k_g_max=m["k_g_max"],
                n_kap=int(m["n_kap"]), n_gam=int(m["n_gam"]), kap_min=m["kap_min"], kap_max=m["kap_max"],
                gam_max=m["gam_max"], xi_min=m["xi_min"], xi_max=m["xi_max"], sigma=m["sigma"],
                phi_at_k_cut=m["phi_at_k_cut"], phi_at_g_cut=m["phi_at_g_cut"])
    if getattr(lam, "xi_coarse_rule", False):
        grid.update(xi_coarse=float(m["xi_coarse"]), xi_coarse_k=float(m["xi_coarse_k"]))
    grid.update(window=float(m["window"]))
    meta = dict(grid=grid, sigma_kappa=sig, mean=m["mean"], var=m["var"], skew=m["skew"], sigmaDL=m["sigmaDL"],
                norm=m["norm"], device_ms=dict(lam=m["ms_lambda"], transforms=m["ms_transform"],
                                               path=m["ms_path"]))
    return xi_out, Ps, meta
