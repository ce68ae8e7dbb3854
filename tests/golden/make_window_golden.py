"""Golden PDF for the positive-definite box window (sgl_full.py:83-94, 254-258), computed by the
REFERENCE's own code.

The stored goldens all have window = 0, so this script makes one with the reference's invert
(sgl_full.py:159-375) and window=True: a 1000-cell subset of the z_s=1 population (seeded choice,
weights scaled so that the total weight is the population's), Psi_1 only.  Without Numba the
reference evaluates Lam with its NumPy dense sum (sgl_full.py:2682-2704), affordable for 1000
cells.  The same population is inverted with window=False as well, so the test sees the window's
effect and not only the PDF.

Writes (committed, small):
  tests/golden/pop_window.npz   -- the population (cells only, no xi groups)
  tests/golden/ref_window.npz   -- invert(...) on the CLI xi grids with window=True and window=False:
                                   P, the grid, the moments and the window flag of each

Usage:  python tests/golden/make_window_golden.py --reference PATH   (or SGL_REFERENCE=PATH; needs
the z_s=1 cells pickle made by make_fixtures.py build)
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
GOLDEN = REPO / "tests" / "golden"
FULL = GOLDEN / "full"
N_CELLS, SEED = 1000, 11
GRID_KEYS = ("nk_k", "nk_g", "k_k_max", "k_g_max", "n_kap", "n_gam", "kap_min", "kap_max", "gam_max",
             "phi_at_k_cut", "phi_at_g_cut", "window")


def main():
    ref = reference_root()
    sys.path.insert(0, str(ref / "src"))
    sys.path.insert(0, str(REPO))
    from sgl_analytic import sgl_full as F          # noqa: E402
    from sgl_analytic_gb300.population import Population
    assert not F._HAVE_NUMBA, "run without numba so the reference uses its NumPy paths"
    pop = Population.load(GOLDEN / "pop_zs1_sub.npz")
    rng = np.random.default_rng(SEED)
    idx = np.sort(rng.choice(pop.w0.size, N_CELLS, replace=False))
    scale = pop.w0.sum() / pop.w0[idx].sum()
    sub = Population(w0=pop.w0[idx] * scale, k0=pop.k0[idx].copy(), g0=pop.g0[idx].copy(),
                     ig=pop.ig[idx].copy(), fe_g=pop.fe_g.copy(), V=pop.V, zs=pop.zs)
    sub.save(GOLDEN / "pop_window.npz")
    with open(FULL / "cells_zs1_gauss.pkl", "rb") as f:
        cells = pickle.load(f)["cells"]
    lam = F.Lam(cells, xi=False, C=None, nord=1, exactS=False, k3=False, q_coarse=101, lss_var=0.0, lam_coarse=0)
    # the reference's compacted cells replaced by the subset (the attributes Lam.__init__ sets)
    lam._ig, lam.w0, lam.k0, lam.g0, lam.V = sub.ig, sub.w0, sub.k0, sub.g0, float(sub.V)
    xo = np.concatenate([np.linspace(-1.0, 1.0, 1601), np.linspace(1.005, 9.0, 1600)])
    out = dict(xi_out=xo, sigma=np.float64(lam.sigma()))
    for tag, win in (("win", True), ("raw", False)):
        t = time.time()
        _, P, meta = F.invert(lam, lam.sigma(), xi_out=xo, tail_box=True, phi_tol=1e-8, nproc=1, window=win,
                              n_xi_wide=500)
        g = meta["grid"]
        print(tag, "invert", time.time() - t, {k: g[k] for k in ("nk_k", "nk_g", "n_kap", "n_gam", "window")},
              flush=True)
        out[tag + "_P"] = P
        out[tag + "_grid"] = np.array([g[k] for k in GRID_KEYS], float)
        out[tag + "_moments"] = np.array([meta["mean"], meta["var"], meta["skew"], meta["sigmaDL"]])
    np.savez_compressed(GOLDEN / "ref_window.npz", **out)


if __name__ == "__main__":
    main()
