"""Golden PDF for the reference's blocked inversion (sgl_full.py:97-157, used above 2e7 k-points).

The reference's ``invert`` switches to ``_invert_blocked`` when nk_k * nk_g > INVERT_BLOCK_PTS.
No stored golden reaches that size, so this script makes one with the reference's own code: a
300-cell subset of the z_s=1 population (seeded choice, weights x 56) whose k-grid is
5267 x 5282 = 2.78e7 points.  Without Numba the reference evaluates Lam with its NumPy dense sum,
which is affordable for 300 cells.

Writes (committed, small):
  tests/golden/pop_blocked.npz  -- the population (cells only, no xi groups)
  tests/golden/ref_blocked.npz  -- invert(...) on the CLI xi grids: P, the grid, the moments

Usage:  python tests/golden/make_blocked_golden.py --reference PATH   (or SGL_REFERENCE=PATH; needs the reference source and the z_s=1
cells pickle made by make_fixtures.py build)
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
N_CELLS, SEED, W_SCALE = 300, 7, 56.0


def subset(pop):
    rng = np.random.default_rng(SEED)
    idx = np.sort(rng.choice(pop.w0.size, N_CELLS, replace=False))
    return idx


def main():
    REF = reference_root()
    sys.path.insert(0, str(REF / "src"))
    sys.path.insert(0, str(REPO))
    from sgl_analytic import sgl_full as F          # noqa: E402
    from sgl_analytic_gb300.population import Population
    assert not F._HAVE_NUMBA, "run without numba so the reference uses its NumPy paths"
    pop = Population.load(GOLDEN / "pop_zs1_sub.npz")
    idx = subset(pop)
    sub = Population(w0=pop.w0[idx] * W_SCALE, k0=pop.k0[idx].copy(), g0=pop.g0[idx].copy(),
                     ig=pop.ig[idx].copy(), fe_g=pop.fe_g.copy(), V=pop.V, zs=pop.zs)
    sub.save(GOLDEN / "pop_blocked.npz")
    with open(FULL / "cells_zs1_gauss.pkl", "rb") as f:
        cells = pickle.load(f)["cells"]
    lam = F.Lam(cells, xi=False, C=None, nord=1, exactS=False, k3=False, q_coarse=101, lss_var=0.0, lam_coarse=0)
    # the reference's compacted cells replaced by the subset (the attributes Lam.__init__ sets)
    lam._ig, lam.w0, lam.k0, lam.g0, lam.V = sub.ig, sub.w0, sub.k0, sub.g0, float(sub.V)
    xo = np.concatenate([np.linspace(-1.0, 1.0, 1601), np.linspace(1.005, 9.0, 1600)])
    t = time.time()
    _, P, meta = F.invert(lam, lam.sigma(), xi_out=xo, tail_box=True, phi_tol=1e-8, nproc=1, window=False,
                          n_xi_wide=500)
    g = meta["grid"]
    assert g["nk_k"] * g["nk_g"] > F.INVERT_BLOCK_PTS, "the case must take the blocked path"
    print("invert", time.time() - t, {k: g[k] for k in ("nk_k", "nk_g", "n_kap", "n_gam")}, flush=True)
    np.savez_compressed(GOLDEN / "ref_blocked.npz", xi_out=xo, P=P, sigma=np.float64(lam.sigma()),
                        grid=np.array([g[k] for k in ("nk_k", "nk_g", "k_k_max", "k_g_max", "n_kap", "n_gam",
                                                      "kap_min", "kap_max", "gam_max")], float),
                        moments=np.array([meta["mean"], meta["var"], meta["skew"], meta["sigmaDL"]]))


if __name__ == "__main__":
    main()
