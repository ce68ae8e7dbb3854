"""vp (positive Cox) closure fixtures from the reference package (run in the development container;
the reference checkout by --reference PATH or SGL_REFERENCE).

Needs the z_s=1 vp cells pickle (built by ``make_fixtures.py build --closure vp`` into tests/golden/full/).
The reference's closure set-up runs UNMODIFIED (under ``oracle/numba_standin``, since
pos_closure_fused imports numba): ``pos_closure.install(lam, cos, "vp")`` (pos_closure.py:708-733)
builds the per-shell cells, the 48-state Gauss-Hermite chain (transition matrices from the
line-of-sight correlations), the rates calibrated to the xi_lin kappa variance (eta), and the
rate-interval parameters of FusedVP (pos_closure_fused.py:18-48).

Writes
  tests/golden/full/vp_zs1_pop.npz   the closure's per-shell population (cells W, kap, gam, phi per
                                      shell; rho, fvar, the kappa / gamma targets; not committed)
  tests/golden/full/vp_zs1_full.npz  the whole closure (67 shells, ~2.45M cells; not committed)
  tests/golden/vp_zs1_sub_pop.npz     shells 0-5 of the per-shell population (committed)
  tests/golden/vp_zs1_sub.npz         shells 0-5 of it (committed) and, computed by the reference's
                                      own _fused_groups + _chain_recursion on that sub-closure,
                                      lnR on a 5 x 4 (k_kappa, k_gamma) grid
  tests/golden/vp_zs1_full_lnR_probe.npz
                                      lnR of the WHOLE closure on a 3 x 3 grid, by the reference's
                                      FusedVP.lnR_blocked ("fused") and Closure.lnR_ref ("ref")
"""
from __future__ import annotations

import pickle
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _reference import reference_root  # noqa: E402

REPO = Path(__file__).resolve().parents[2]
STANDIN = REPO / "oracle" / "numba_standin"
NSUB = 6


def main():
    REF_SRC = reference_root() / "src"
    for p in (str(REF_SRC), str(STANDIN)):
        sys.path.insert(0, p)
    from scipy.special import j0
    from sgl_analytic import pipeline as PL, pos_closure as PC, sgl_full as F
    with open(REPO / "tests" / "golden" / "full" / "cells_zs1_vp.pkl", "rb") as f:
        cells = pickle.load(f)["cells"]
    cos = PL.make_cosmology(None)
    t = time.time()
    lam = F.Lam(cells, C=None, nord=1, exactS=False, k3=False, xi=True)
    pos = PC.install(lam, cos, kind="vp")
    print("install", time.time() - t, pos.eval_kernel, "eta", pos.eta, flush=True)
    # the closure's per-shell population (pos_closure.population, pos_closure.py:388-450): the input
    # of the closure set-up (Closure.__init__, calibrate, the rate intervals), which the engine
    # restates; its output is the closure saved below
    pp = pos.pop
    cl = pp["cells"]
    np.savez_compressed(REPO / "tests" / "golden" / "full" / "vp_zs1_pop.npz",
                        shell_start=np.concatenate([[0], np.cumsum([c["W"].size for c in cl])]).astype(np.int64),
                        W=np.concatenate([c["W"] for c in cl]), kap=np.concatenate([c["kap"] for c in cl]),
                        gam=np.concatenate([c["gam"] for c in cl]), phi=np.concatenate([c["phi"] for c in cl]),
                        rho=np.asarray(pp["rho"], float), fvar=np.asarray(pp["fvar"], float),
                        target_kappa=np.float64(pp["target_kappa"]), target_gamma=np.float64(pp["target_gamma"]),
                        eta=np.float64(pos.eta))
    # shells 0 .. NSUB-1 of that population (committed): the input of the set-up for the sub-closure
    # below, which uses the whole closure's eta
    c1p = int(np.sum([c["W"].size for c in cl[:NSUB]]))
    np.savez_compressed(REPO / "tests" / "golden" / "vp_zs1_sub_pop.npz",
                        shell_start=np.concatenate([[0], np.cumsum([c["W"].size for c in cl[:NSUB]])]).astype(np.int64),
                        W=np.concatenate([c["W"] for c in cl[:NSUB]]), kap=np.concatenate([c["kap"] for c in cl[:NSUB]]),
                        gam=np.concatenate([c["gam"] for c in cl[:NSUB]]), phi=np.concatenate([c["phi"] for c in cl[:NSUB]]),
                        rho=np.asarray(pp["rho"][:NSUB - 1], float), fvar=np.asarray(pp["fvar"][:NSUB], float),
                        target_kappa=np.float64(pp["target_kappa"]), target_gamma=np.float64(pp["target_gamma"]),
                        eta=np.float64(pos.eta), n_cells=np.int64(c1p))
    fused = pos.lnR_blocked.__self__               # the FusedVP instance
    B = pos._B
    full = dict(u=pos.u, w=pos.w, K=pos._Karr, shear_var=np.float64(pos.shear_var), eta=np.float64(pos.eta),
                ku=pos.ku, gu=pos.gu, cu=B["cu"].astype(np.int32), cw=B["cw"], gstart=B["gstart"],
                sh_g=B["sh_g"], ga=fused.a, gb=fused.b, gc=fused.c, glo=fused.lo.astype(np.int32),
                ghi=fused.hi.astype(np.int32), sigma=np.float64(lam.sigma()))
    np.savez_compressed(REPO / "tests" / "golden" / "full" / "vp_zs1_full.npz", **full)
    # --- sub-closure: shells 0 .. NSUB-1
    sh_g, gstart = B["sh_g"], B["gstart"]
    g1 = int(sh_g[NSUB])
    c1 = int(gstart[g1])
    cu = B["cu"][:c1]
    used, cu_new = np.unique(cu, return_inverse=True)
    sub = dict(u=pos.u, w=pos.w, K=pos._Karr[:NSUB - 1], shear_var=np.float64(pos.shear_var),
               ku=pos.ku[used], gu=pos.gu[used], cu=cu_new.astype(np.int32), cw=B["cw"][:c1],
               gstart=gstart[:g1 + 1], sh_g=sh_g[:NSUB + 1], ga=fused.a[:g1], gb=fused.b[:g1], gc=fused.c[:g1],
               glo=fused.lo[:g1].astype(np.int32), ghi=fused.hi[:g1].astype(np.int32))
    kv = np.array([0.0, 3.0, 40.0, 250.0, 900.0])
    qv = np.array([0.0, 20.0, 150.0, 600.0])
    from sgl_analytic import pos_closure_fused as PF
    e = np.expm1(1j * np.outer(sub["ku"], kv))
    J = np.ascontiguousarray(j0(np.outer(sub["gu"], qv)))
    P = kv.size * qv.size
    zr = np.empty((NSUB, pos.w.size, P)); zi = np.empty_like(zr)
    t = time.time()
    PF._fused_groups(np.ascontiguousarray(e.real), np.ascontiguousarray(e.imag), J, J - 1.0,
                     sub["cu"].astype(np.int64), sub["cw"], sub["gstart"].astype(np.int64), sub["sh_g"].astype(np.int64),
                     sub["ga"], sub["gb"], sub["gc"], sub["glo"].astype(np.int64), sub["ghi"].astype(np.int64),
                     pos.u, zr, zi)
    r, i = PC._chain_recursion(zr, zi, sub["K"], pos.w)
    print("reference sub-closure lnR", time.time() - t, flush=True)
    sub.update(kv=kv, qv=qv, lnR=(r + 1j * i).reshape(kv.size, qv.size))
    np.savez_compressed(REPO / "tests" / "golden" / "vp_zs1_sub.npz", **sub)
    print("sub cells", c1, "groups", g1, "unique", used.size)
    kv3, qv3 = np.array([0.0, 37.0, 400.0]), np.array([0.0, 55.0, 300.0])
    t = time.time()
    fz = pos.lnR_blocked(kv3, qv3)
    rf = pos.lnR_ref(kv3, qv3)
    print("full-closure probe", time.time() - t, "max |fused - ref|", float(np.abs(fz - rf).max()), flush=True)
    np.savez(REPO / "tests" / "golden" / "vp_zs1_full_lnR_probe.npz", kv=kv3, qv=qv3, fused=fz, ref=rf)


if __name__ == "__main__":
    main()
