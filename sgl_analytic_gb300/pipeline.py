"""Drop-in orchestration: the reference's ``pipeline.run`` with the hot path on the GPU.

``run(zs, cfg, ...)`` validates its arguments exactly as the reference does (sgl_analytic
pipeline.py:36-164; the cosmology domain of sgl.py:111-151), then

  1. population build (L2, upstream of the hot path): the reference package's own CPU builder
     when ``sgl_analytic`` is importable, or a pre-built ``population=`` (a ``Population`` or a
     population ``.npz``);
  2. ``Lam`` + ``invert`` on the GPU (this package);
  3. the reference's output dict (pipeline.py:243-271) for the keys the hot path determines.

Only the default chain is on the GPU path: clustering "xilin" with the gauss or the vp closure, edge
"r200" or "rvir".  Everything else raises ``NotImplementedError`` (there is no CPU fallback).  The vp
closure's set-up (shells, chain, rates) comes with the population: a pre-built population carries it
(``Population.vp``), a population built here gets it from the reference package.
"""
from __future__ import annotations

import time
import warnings
from pathlib import Path

import numpy as np

P = dict(h=0.674, Om=0.315, s8=0.811, Ob=0.0493, ns=0.965, zeq=3402.0)
EXTENSIONS = dict(Ok=0.0, w0=-1.0, wa=0.0, growth_mode="ode", radiation="engine")
INGREDIENTS = ("ell", "fil", "sub", "bias")
DE_REC_CAP = 1e-2
# the fine (kappa, gamma) lattice of the population build (sgl_full.py:456): (lo, hi, bins per sign)
FINE = dict(k=(1e-7, 30.0, 480), g=(1e-9, 30.0, 300))


def on(cfg):
    """Lens ingredients switched on (reference pipeline.py:78-94)."""
    ing = set(INGREDIENTS)
    if not isinstance(cfg, str):
        s = set(cfg)
        if s - ing:
            raise ValueError(f"unknown ingredient(s) {sorted(s - ing)}; choose from {INGREDIENTS}")
        return s
    if cfg == "halo":
        return set()
    if cfg == "full":
        return ing
    if len(cfg) < 2 or cfg[0] not in "+-" or cfg[1:] not in ing:
        raise ValueError(f"unknown configuration {cfg!r}; use full, halo, or +/-{INGREDIENTS}")
    return {cfg[1:]} if cfg[0] == "+" else ing - {cfg[1:]}


def cfg_name(cfg):
    if isinstance(cfg, str):
        return cfg
    s = on(cfg)
    return "full" if s == set(INGREDIENTS) else ("halo" if not s else
                                                 "halo+" + "+".join(i for i in INGREDIENTS if i in s))


def cosmology_params(cosmo=None):
    """Validated cosmology parameters (reference make_cosmology, pipeline.py:36-72, plus the
    Cosmology domain checks of sgl.py:111-151).  Returns the complete parameter dict."""
    supplied = dict(cosmo or {})
    if "sigma8" in supplied:
        if "s8" in supplied:
            raise ValueError("supply sigma8 or s8, not both")
        supplied["s8"] = supplied.pop("sigma8")
    cp = {**P, **EXTENSIONS, **supplied}
    bad = set(cp) - set(P) - set(EXTENSIONS)
    if bad:
        raise ValueError(f"unknown cosmology parameter(s) {sorted(bad)}")
    for key in P:
        v = cp[key]
        if not np.isscalar(v) or not np.isfinite(v) or v <= 0:
            raise ValueError(f"{key} must be a finite positive number")
    for key in ("Ok", "w0", "wa"):
        v = cp[key]
        if isinstance(v, bool) or not np.isscalar(v) or not np.isfinite(v):
            raise ValueError(f"{key} must be a finite number")
    if cp["growth_mode"] not in ("auto", "ode", "legacy"):
        raise ValueError("growth_mode must be 'auto', 'ode' or 'legacy'")
    if cp["radiation"] in ("none", False):
        cp["radiation"] = None
    if cp["radiation"] not in ("engine", None):
        raise ValueError("radiation must be 'engine' or None")
    if not 0 < cp["Ob"] < cp["Om"] <= 1:
        raise ValueError("require 0 < Ob < Om <= 1")
    w0, wa, Om, Ok = float(cp["w0"]), float(cp["wa"]), float(cp["Om"]), float(cp["Ok"])
    Or = Om / (1.0 + float(cp["zeq"])) if cp["radiation"] == "engine" else 0.0
    OL = 1.0 - Om - Ok - Or
    if not -2.0 <= w0 <= 1.0:
        raise ValueError("dark energy requires -2 <= w0 <= 1")
    if w0 + wa >= 0.0:
        raise ValueError("dark energy requires w0 + wa < 0 (matter-dominated early universe)")
    z = 1100.0
    if OL / Om * (1 + z) ** (3 * (w0 + wa)) * np.exp(-3 * wa * z / (1 + z)) > DE_REC_CAP:
        raise ValueError("dark energy exceeds 1e-2 of the matter density at z = 1100")
    lam = w0 == -1.0 and wa == 0.0
    if cp["growth_mode"] == "legacy" and not lam:
        raise ValueError("legacy growth is only valid for LambdaCDM")
    a = np.geomspace(1e-6, 1.0, 4096)
    zp1 = 1.0 / a
    e2 = Om * zp1 ** 3 + Or * zp1 ** 4 + Ok * zp1 ** 2 + OL * zp1 ** (3 * (1 + w0 + wa)) * np.exp(-3 * wa * (1 - a))
    if not np.all(e2 > 0):
        raise ValueError("E(z)^2 <= 0 somewhere in 0 <= z <= 1e6: outside the supported (non-bouncing) domain")
    return cp


def make_cosmology(cosmo=None):
    """The reference's Cosmology object (needed only by the CPU population build)."""
    cp = cosmology_params(cosmo)
    from sgl_analytic import pipeline as ref_pipeline      # the reference package (population build)
    return ref_pipeline.make_cosmology({k: (v if k != "radiation" else (v or "none")) for k, v in cp.items()})


def _load_population(population):
    from .population import Population
    if isinstance(population, Population):
        return population
    return Population.load(Path(population))


def run(zs, cfg="full", nord=4, grid_scale=1.0, xi_out=None, split=10.0, exact_s=True, k3=True, nproc=1,
        sub_kw=None, s_taper="cos2", cosmo=None, tail_box=True, xi_tail=None, s_is=True, s_seed=None,
        q_coarse=101, clustering="xilin", edge="r200", kap_floor=1e-8, phi_tol=1e-8, lam_coarse=0,
        zint="midpoint", zint_n=2, xi_kw=None, xi_closure="gauss", window=None, n_xi_wide=None, keep=False,
        population=None, precision="fp64", device=0):
    """Reference pipeline.run (pipeline.py:114-274) with the Lam/invert stages on the GPU."""
    if clustering in ("linear", "limber", "xilin"):
        nord, k3, exact_s = 1, False, False
    elif clustering != "closure":
        raise ValueError(f"clustering must be 'xilin', 'linear', 'limber' or 'closure', got {clustering!r}")
    if not np.isscalar(zs) or not np.isfinite(zs) or zs <= 0:
        raise ValueError("z_s must be a finite positive number")
    if isinstance(nproc, bool) or not isinstance(nproc, (int, np.integer)) or nproc < 1:
        raise ValueError("nproc must be a positive integer")
    if edge not in ("r200", "rvir", "kthr"):
        raise ValueError("edge must be 'r200', 'rvir' or 'kthr'")
    if xi_closure not in ("gauss", "vp"):
        raise ValueError(f"xi_closure must be 'gauss' or 'vp', got {xi_closure!r}")
    s = on(cfg)
    use_xi = clustering == "xilin" and "bias" in s
    if use_xi and edge == "kthr":
        raise ValueError("clustering='xilin' needs edge='r200' or 'rvir'")
    if xi_closure != "gauss" and not use_xi:
        raise ValueError(f"xi_closure={xi_closure!r} needs xilin clustering and the bias ingredient")
    cp = cosmology_params(cosmo)
    if clustering != "xilin" or edge == "kthr" or grid_scale != 1.0 or lam_coarse:
        raise NotImplementedError("only the default chain (clustering='xilin', edge r200/rvir) is on the GPU path")
    if {**EXTENSIONS, **(cosmo or {})}["growth_mode"] == "auto" and not (cp["w0"] == -1.0 and cp["wa"] == 0.0):
        warnings.warn("growth_mode='auto' resolved to 'ode' for non-Lambda dark energy, while Lambda runs under "
                      "'auto' use the historical growth; compare against a growth_mode='ode' Lambda run.",
                      stacklevel=2)
    from .lam import Lam, invert
    t0 = time.time()
    info = {}
    if population is not None:
        pop = _load_population(population)
        if xi_closure != "gauss" and pop.vp is None:
            raise ValueError(f"xi_closure={xi_closure!r} needs a population that carries its closure (Population.vp)")
    else:
        pop, info = _build_population_with_reference(zs, cfg, s, cp, sub_kw, split, edge, kap_floor, zint, zint_n,
                                                     xi_kw, use_xi, nproc, nord, xi_closure)
    t_build = time.time()
    lam = Lam(pop, C=None, nord=nord, exactS=False, k3=False, s_taper=s_taper, q_coarse=q_coarse, xi=use_xi,
              precision=precision, device=device)
    pos_info = None
    if xi_closure != "gauss":
        # the positive closure replaces the gauss term (pos_closure.install, pipeline.py:206-209)
        t_pos = time.time()
        lam.install_vp(pop.vp)
        pos_info = dict(kind=xi_closure, eta=(float(pop.vp["eta"]) if "eta" in pop.vp else None),
                        nstate=int(np.asarray(pop.vp["u"]).size), shells=int(np.asarray(pop.vp["sh_g"]).size - 1),
                        eval_kernel="gpu", setup_seconds=info.get("pos_setup_seconds", 0.0) + time.time() - t_pos,
                        lnR_seconds=None)
    sig = lam.sigma()
    t_lam = time.time()
    if xi_out is None:
        xi_out = np.linspace(-1.0, 1.0, 1601)
        if xi_tail is None:
            xi_tail = np.linspace(1.005, 9.0, 1600)
    nx = len(xi_out)
    xall = np.asarray(xi_out, float) if xi_tail is None else np.concatenate([xi_out, xi_tail])
    # window=None: "auto" for a positive closure, False for gauss; n_xi_wide=None: 500 for gauss,
    # 4000 otherwise (reference pipeline.py:216-231)
    if window is None:
        window = "auto" if xi_closure != "gauss" else False
    if window not in (False, True, "auto"):
        raise ValueError(f"window must be True, False, 'auto' or None, got {window!r}")
    if n_xi_wide is None:
        n_xi_wide = 500 if xi_closure == "gauss" else 4000
    xa, Pa, meta = invert(lam, sig, xi_out=xall, tail_box=tail_box, phi_tol=phi_tol, nproc=1, window=window,
                          n_xi_wide=n_xi_wide)
    t_inv = time.time()
    # every key of the reference's output dict (pipeline.py:243-271); the ones the population build
    # determines come from it when it ran here, None when the population was given
    Or = cp["Om"] / (1.0 + cp["zeq"]) if cp["radiation"] == "engine" else 0.0
    out = dict(t_stages=dict(build=t_build - t0, lam=t_lam - t_build, invert=t_inv - t_lam), zs=zs,
               cfg=cfg_name(cfg), zint=zint, zint_n=(zint_n if zint == "gauss" else None), clustering=clustering,
               xi_kperp=info.get("xi_kperp"), edge=edge, lss_var=0.0, kap_floor=(kap_floor if edge != "kthr" else None),
               kbar=info.get("kbar"), h=cp["h"], Om=cp["Om"], s8=cp["s8"], Ob=cp["Ob"], ns=cp["ns"], zeq=cp["zeq"],
               sigma8=cp["s8"], Ok=cp["Ok"], w0=cp["w0"], wa=cp["wa"], growth_mode=cp["growth_mode"],
               radiation=cp["radiation"], Omega_r=Or, nord=nord, grid_scale=grid_scale, split=split, nproc=nproc,
               sub_kw=info.get("sub_kw"), pair_angle=info.get("pair_angle"), k3=False, exactS=False,
               s_taper=s_taper, sigma_kappa=sig, kthr=None, N_expl=info.get("N_expl"),
               N_fil=info.get("N_fil"), V_weak=info.get("V_weak"), mean=meta["mean"], var=meta["var"],
               skew=meta["skew"], sigmaDL=meta["sigmaDL"],
               grid={k: v for k, v in meta["grid"].items() if isinstance(v, (int, float))},
               tail_box=bool(tail_box), fine=dict(FINE), s_is=bool(s_is), xi_closure=xi_closure, window=window,
               n_xi_wide=n_xi_wide, pos_closure=pos_info, direct_product_backend="unused",
               s_seed=(int(s_seed) if s_seed is not None else None), s_seed_effective=(int(s_seed) if s_seed is not None
                                                                                       else 0),
               s_ess=None, is_design=None, engine=dict(precision=precision, device_ms=meta["device_ms"]),
               seconds=time.time() - t0, xi=np.asarray(xa[:nx]).tolist(), P_s=np.asarray(Pa[:nx]).tolist())
    if xi_tail is not None:
        out.update(xi_tail=np.asarray(xa[nx:]).tolist(), P_s_tail=np.asarray(Pa[nx:]).tolist())
    meta_out = dict(meta)
    if keep:
        meta_out.update(population=pop, lam=lam, info=info)
    return out, meta_out


def _build_population_with_reference(zs, cfg, s, cp, sub_kw, split, edge, kap_floor, zint, zint_n, xi_kw, use_xi,
                                     nproc, nord, xi_closure="gauss"):
    """The population build (upstream of the hot path) through the reference package; for a
    positive closure also the closure's set-up (pos_closure.install on the reference's own Lam,
    pos_closure.py:708-733), whose arrays the GPU Lam then takes."""
    try:
        from sgl_analytic import sgl_full as F
        from sgl_analytic import subhalos
    except ImportError as exc:
        raise RuntimeError("the population build needs the reference package sgl_analytic (or pass population=)") \
            from exc
    from .population import Population
    cos = make_cosmology({k: v for k, v in cp.items()})
    trunc = "r200" if edge == "r200" else "rvir"
    skw = dict(sector="exact", clump_edge=trunc, exact_kw=dict(method="moments"))
    skw.update(sub_kw or {})
    sub = subhalos.SubhaloModel(cos, zs, None, split=split, **skw) if "sub" in s else None
    xi = F.xi_kperp_grid(cos, **(xi_kw or {})) if use_xi else None
    if xi is not None and xi_closure != "gauss":
        xi["pos"] = True
    cells, info = F.build_population(cos, zs, ell="ell" in s, fils="fil" in s, nord=nord, kthr=None, subhalo=sub,
                                     nproc=nproc, zint=zint, zint_n=zint_n, xi=xi, kap_floor=kap_floor, trunc=trunc)
    pop = Population.from_cells(cells)
    pop.zs = float(zs)
    info = dict(info)
    info["xi_kperp"] = {k: xi[k] for k in ("kmin", "kmax", "per_decade", "mmax")} if xi else None
    info["sub_kw"] = sub._init_kw if sub is not None else None
    info["pair_angle"] = sub.pair_angle if sub is not None else None
    if xi_closure != "gauss":
        import time as _time
        from sgl_analytic import pos_closure
        t = _time.time()
        ref_lam = F.Lam(cells, C=None, nord=1, exactS=False, k3=False, xi=True)
        pos = pos_closure.install(ref_lam, cos, kind=xi_closure)
        pop.vp = closure_arrays(pos)
        info["pos_setup_seconds"] = _time.time() - t
    return pop, info


def closure_arrays(pos):
    """The arrays of a reference closure object (pos_closure.install's return; its FusedVP rate
    intervals, pos_closure_fused.py:18-48) in the form Lam.install_vp takes."""
    fused = pos.lnR_blocked.__self__
    B = pos._B
    return dict(u=pos.u, w=pos.w, K=pos._Karr, shear_var=float(pos.shear_var), eta=float(pos.eta), ku=pos.ku,
                gu=pos.gu, cu=B["cu"].astype(np.int32), cw=B["cw"], gstart=B["gstart"], sh_g=B["sh_g"], ga=fused.a,
                gb=fused.b, gc=fused.c, glo=fused.lo.astype(np.int32), ghi=fused.hi.astype(np.int32))


def clipped_moments(xi, P, clip=1.0):
    """Moments of the PDF restricted to |xi| <= clip (reference pipeline.py:277-284)."""
    m = np.abs(xi) <= clip
    x, p = xi[m], P[m]
    p = p / np.trapezoid(p, x)
    mu = np.trapezoid(x * p, x)
    v = np.trapezoid((x - mu) ** 2 * p, x)
    return dict(mean=float(mu), var=float(v), skew=float(np.trapezoid((x - mu) ** 3 * p, x) / v ** 1.5))
