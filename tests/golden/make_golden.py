"""Golden vectors for the GPU parity tests, computed by the REFERENCE's own code.

Run in the development container (needs the reference source and the z_s=1 cells pickle made by
``make_fixtures.py build``).  Without Numba the reference's ``Lam`` evaluates every grid with its
pure-NumPy dense sum ``_lam_worker_block`` (sgl_full.py:2682-2704) and its NumPy ``_Qxi_gauss``
(sgl_full.py:2869-2951); ``invert`` (sgl_full.py:159-375) is NumPy/SciPy throughout.

Writes (committed, a few MB):
  tests/golden/pop_zs1_sub.npz  -- population: all 79,574 occupied fine cells of the reference's
                                   z_s=1 build + the three xi_lin groups (m = 0, 1, 2) of shell 30
  tests/golden/ref_zs1_sub.npz  -- reference outputs on that population:
       psi1_*   Lam(xi=False) on a 53 x 84 subgrid of the z_s=1 inversion grid and on the
                k-reach probe axes
       xi_*     Lam(xi=True)._Qxi_gauss on the 101^2 coarse grid and the probe axes
       pdf1_*   invert(Lam(xi=False)) on the CLI xi grids (1601 + 1600 points)
       pdfx_*   invert(Lam(xi=True))  on the same grids
Also copies the reference's stored golden PDFs (tests/reference/pdf_zs*.json) next to them.

Usage:  python tests/golden/make_golden.py --reference PATH   (or SGL_REFERENCE=PATH)
"""
from __future__ import annotations

import pickle
import shutil
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _reference import reference_root  # noqa: E402

REPO = Path(__file__).resolve().parents[2]
GOLDEN = REPO / "tests" / "golden"
FULL = REPO / "tests" / "golden" / "full"          # large, git-ignored
WORK = FULL
SHELL = 30


def main():
    REF = reference_root()
    sys.path.insert(0, str(REF / "src"))
    sys.path.insert(0, str(REPO))
    from sgl_analytic import sgl_full as F          # noqa: E402  (no numba: NumPy paths)
    from sgl_analytic_gb300.population import Population
    assert not F._HAVE_NUMBA, "run without numba so the reference uses its NumPy paths"
    for p in sorted((REF / "tests" / "reference").glob("pdf_zs*.json")):
        shutil.copy(p, GOLDEN / p.name)
    with open(WORK / "cells_zs1_gauss.pkl", "rb") as f:
        cells = pickle.load(f)["cells"]
    groups_all = cells.xi_groups
    sel = [i for i, g in enumerate(groups_all) if int(g["shell"]) == SHELL]
    cells.xi_groups = [groups_all[i] for i in sel]
    pop = Population.from_cells(cells)
    pop.zs = 1.0
    pop.save(GOLDEN / "pop_zs1_sub.npz")

    kw = dict(C=None, nord=1, exactS=False, k3=False, q_coarse=101, lss_var=0.0, lam_coarse=0)
    lam1 = F.Lam(cells, xi=False, **kw)
    lamx = F.Lam(cells, xi=True, **kw)
    out = dict(groups=np.array(sel), shell=np.int64(SHELL))
    # subgrid of the z_s=1 inversion grid (tests/reference/pdf_zs1.json grid)
    kk = np.linspace(0.0, 1010.4632803971984, 1683)[::32]
    kg = np.linspace(0.0, 808.3706243177588, 2687)[::32]
    out.update(kk=kk, kg=kg)
    t = time.time()
    out["psi1_grid"] = lam1(kk, kg)
    sig1 = lam1.sigma()
    ks = (12.0 / sig1) * 1.25 ** np.arange(20)
    out.update(probe_k=ks, psi1_line_k=lam1(ks, np.zeros(1))[:, 0], psi1_line_g=lam1(np.zeros(1), ks)[0, :],
               sigma1=np.float64(sig1))
    sigx = lamx.sigma()
    s = np.linspace(0.0, 1.0, 101)
    kkc, kgc = kk[-1] * s ** 2, kg[-1] * s ** 2
    out.update(kkc=kkc, kgc=kgc, xi_coarse=lamx._Qxi_gauss(kkc, kgc), sigmax=np.float64(sigx),
               xi_line_k=lamx._Qxi_gauss(ks, np.zeros(1))[:, 0], xi_line_g=lamx._Qxi_gauss(np.zeros(1), ks)[0, :],
               lamx_grid=lamx(kk[:20], kg[:20]))
    print("lam parts", time.time() - t, flush=True)
    xo = np.concatenate([np.linspace(-1.0, 1.0, 1601), np.linspace(1.005, 9.0, 1600)])
    out["xi_out"] = xo
    for tag, lam in (("pdf1", lam1), ("pdfx", lamx)):
        t = time.time()
        _, P, meta = F.invert(lam, lam.sigma(), xi_out=xo, tail_box=True, phi_tol=1e-8, nproc=1, window=False,
                              n_xi_wide=500)
        g = meta["grid"]
        out[tag + "_P"] = P
        out[tag + "_grid"] = np.array([g[k] for k in ("nk_k", "nk_g", "k_k_max", "k_g_max", "n_kap", "n_gam",
                                                      "kap_min", "kap_max", "gam_max", "phi_at_k_cut",
                                                      "phi_at_g_cut")], float)
        out[tag + "_moments"] = np.array([meta["mean"], meta["var"], meta["skew"], meta["sigmaDL"]])
        print(tag, "invert", time.time() - t, {k: g[k] for k in ("nk_k", "nk_g", "n_kap", "n_gam")}, flush=True)
    np.savez_compressed(GOLDEN / "ref_zs1_sub.npz", **out)


if __name__ == "__main__":
    main()
