"""Generate the golden fixtures from the reference package (run in the development container).

The reference (sgl_analytic v0.2.0) is pure Python + NumPy/SciPy + Numba.  Numba is not
installable here, so this script puts ``oracle/numba_standin`` (``njit`` = identity,
``prange`` = range) first on ``sys.path`` and runs the reference source UNMODIFIED.

Stage ``build`` (slow, ~30 min per z_s on 8 cores): replicates ``pipeline.run`` up to the
population build (sgl_analytic/pipeline.py:165-192) and pickles the reference's own
``Cells`` object into ``tests/golden/full/`` (large, git-ignored, never committed).

Stage ``extract``: from the pickle, constructs the reference ``Lam`` (sgl_full.py:2728) and
writes the compact inputs of the hot path -- the occupied fine cells (w0, k0, g0, fine gamma
bin), the weak-arm variance, the xi_lin groups and the coarse lattice centres -- plus
the reference's sigma.  Output: ``tests/golden/full/cells_zs<z>_<closure>_full.npz`` (all xi groups;
~290 MB at z_s=1, not committed; the committed subset is made by ``make_golden.py``).

Usage (from the repository root; the reference checkout by --reference PATH or SGL_REFERENCE)::

    python tests/golden/make_fixtures.py build   --zs 1 --closure gauss --nproc 8 --reference PATH
    python tests/golden/make_fixtures.py extract --zs 1 --closure gauss --reference PATH
"""
from __future__ import annotations

import argparse
import os
import pickle
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _reference import reference_root, strip_reference_args  # noqa: E402

REPO = Path(__file__).resolve().parents[2]
STANDIN = REPO / "oracle" / "numba_standin"
FULL = REPO / "tests" / "golden" / "full"          # large, git-ignored
WORK = FULL
GOLDEN = REPO / "tests" / "golden"


def _setup_path():
    REF_SRC = reference_root() / "src"
    for p in (str(REF_SRC), str(STANDIN)):
        if p not in sys.path:
            sys.path.insert(0, p)
    # spawned build workers inherit the environment, not sys.path
    os.environ["PYTHONPATH"] = os.pathsep.join([str(STANDIN), str(REF_SRC)]
                                               + [os.environ.get("PYTHONPATH", "")])


def _tag(zs, closure):
    return f"zs{zs:g}_{closure}"


def build(zs, closure, nproc):
    _setup_path()
    from sgl_analytic import pipeline as PL, sgl_full as F, subhalos
    cos = PL.make_cosmology(None)
    skw = dict(sector="exact", clump_edge="r200", exact_kw=dict(method="moments"))
    t0 = time.time()
    sub = subhalos.SubhaloModel(cos, zs, None, split=10.0, **skw)
    xi = F.xi_kperp_grid(cos)
    if closure != "gauss":
        xi["pos"] = True
    cells, info = F.build_population(cos, zs, ell=True, fils=True, nord=1, kthr=None,
                                     subhalo=sub, nproc=nproc, zint="midpoint", zint_n=2,
                                     xi=xi, kap_floor=1e-8, trunc="r200")
    t1 = time.time()
    WORK.mkdir(parents=True, exist_ok=True)
    with open(WORK / f"cells_{_tag(zs, closure)}.pkl", "wb") as f:
        pickle.dump(dict(cells=cells, info=info, xi=xi, build_seconds=t1 - t0), f,
                    protocol=pickle.HIGHEST_PROTOCOL)
    print(f"build {t1 - t0:.1f} s", flush=True)


def extract(zs, closure):
    _setup_path()
    from sgl_analytic import sgl_full as F
    with open(WORK / f"cells_{_tag(zs, closure)}.pkl", "rb") as f:
        d = pickle.load(f)
    cells = d["cells"]
    lam = F.Lam(cells, C=None, nord=1, exactS=False, k3=False, s_taper="cos2", s_is=True,
                q_coarse=101, lss_var=0.0, lam_coarse=0, xi=True)
    sig = lam.sigma()
    out = dict(w0=lam.w0, k0=lam.k0, g0=lam.g0, ig=lam._ig.astype(np.int32),
               fe_g=cells.fe[1], V=np.float64(lam.V), sigma=np.float64(sig),
               ce_k=cells.ce[0], ce_g=cells.ce[1], zs=np.float64(zs))
    # raw xi_lin groups (before Lam's xi_prune): m, idx, rows, concatenated
    gs = cells.xi_groups
    out["xg_m"] = np.array([int(g["m"]) for g in gs], np.int32)
    out["xg_shell"] = np.array([int(g["shell"]) for g in gs], np.int32)
    out["xg_nidx"] = np.array([g["idx"].size for g in gs], np.int64)
    out["xg_nrow"] = np.array([g["rows"].shape[0] for g in gs], np.int64)
    out["xg_idx"] = np.concatenate([g["idx"] for g in gs]).astype(np.int32)
    out["xg_rows"] = np.concatenate([g["rows"].ravel() for g in gs])
    FULL.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(FULL / f"cells_{_tag(zs, closure)}_full.npz", **out)
    print("cells", lam.w0.size, "groups", len(gs), "rows", int(out["xg_nrow"].sum()),
          "row-values", out["xg_rows"].size, "sigma", sig, flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("stage", choices=("build", "extract"))
    ap.add_argument("--zs", type=float, default=1.0)
    ap.add_argument("--closure", default="gauss", choices=("gauss", "vp"))
    ap.add_argument("--nproc", type=int, default=os.cpu_count())
    a = ap.parse_args(strip_reference_args(sys.argv[1:]))
    if a.stage == "build":
        build(a.zs, a.closure, a.nproc)
    else:
        extract(a.zs, a.closure)


if __name__ == "__main__":
    main()
