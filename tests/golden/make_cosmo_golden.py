"""Golden cosmology tables computed by the REFERENCE's own Cosmology (sgl.py:65-640), as the chain builds
it (pipeline.make_cosmology, pipeline.py:39-79: EH98 transfer, smooth-k sigma(M) window, top-hat sigma_8
anchor, Ludlow+16 concentrations, ODE growth, radiation Omega_r = Om / (1 + z_eq)).

Cosmologies: the default Planck one and seeded draws over the batched-sweep box (h, Om, sigma8, Ob, ns,
Ok, w0, wa), plus curvature and CPL corners.  For each: E(z), the radial comoving distance chi(z) [Mpc],
the transverse D_M(z), the growth D(z) at the z grid; sigma(M) at z = 0, d ln sigma / d ln M and the
Sheth-Tormen dn/dln M (M, z) at the M grid; the concentration (M, z); Sigma_cr(z_l, z_s) on a few pairs.

Writes tests/golden/cosmo_ref.npz (committed, small).

Usage:  python tests/golden/make_cosmo_golden.py --reference PATH   (or SGL_REFERENCE=PATH)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _reference import reference_root  # noqa: E402

REPO = Path(__file__).resolve().parents[2]
Z = np.array([0.0, 0.01, 0.1, 0.25, 0.5, 0.75, 1.0, 1.5, 2.0, 3.0, 4.5, 6.0, 8.0, 10.0])
M = np.geomspace(1e6, 1e16, 41)
Z_MF = np.array([0.0, 0.5, 1.0, 3.0])
PAIRS = np.array([[0.1, 1.0], [0.5, 1.0], [0.3, 3.0], [2.0, 10.0]])
KEYS = ("h", "Om", "Ob", "s8", "ns", "zeq", "Ok", "w0", "wa")


def cosmologies():
    rng = np.random.default_rng(7)
    out = [dict(h=0.674, Om=0.315, Ob=0.0493, s8=0.811, ns=0.965, zeq=3402.0, Ok=0.0, w0=-1.0, wa=0.0),
           dict(h=0.674, Om=0.315, Ob=0.0493, s8=0.811, ns=0.965, zeq=3402.0, Ok=0.05, w0=-1.0, wa=0.0),
           dict(h=0.674, Om=0.315, Ob=0.0493, s8=0.811, ns=0.965, zeq=3402.0, Ok=-0.05, w0=-0.8, wa=-0.4)]
    box = np.array([[0.6, 0.8], [0.2, 0.4], [0.7, 0.9], [0.04, 0.06], [0.92, 1.0], [-0.05, 0.05], [-1.3, -0.7],
                    [-0.5, 0.5]])
    while len(out) < 9:
        u = box[:, 0] + rng.random(8) * (box[:, 1] - box[:, 0])
        c = dict(h=u[0], Om=u[1], s8=u[2], Ob=u[3], ns=u[4], zeq=3402.0, Ok=u[5], w0=u[6], wa=u[7])
        if c["w0"] + c["wa"] < -0.05:
            out.append(c)
    return out


def main():
    ref = reference_root()
    sys.path.insert(0, str(ref / "src"))
    from sgl_analytic import pipeline as PL          # noqa: E402
    rows = {k: [] for k in ("params", "E", "chi", "DM", "D", "sigmaM", "dlnsig", "dndlnM", "conc", "Sigma_cr")}
    for c in cosmologies():
        cos = PL.make_cosmology(dict(h=c["h"], Om=c["Om"], s8=c["s8"], Ob=c["Ob"], ns=c["ns"], zeq=c["zeq"],
                                     Ok=c["Ok"], w0=c["w0"], wa=c["wa"]))
        rows["params"].append([c[k] for k in KEYS])
        rows["E"].append([float(cos.E(z)) for z in Z])
        rows["chi"].append([cos.chi(z) for z in Z])
        rows["DM"].append([cos.DM(z) for z in Z])
        rows["D"].append([cos.D(z) for z in Z])
        rows["sigmaM"].append(cos.sigmaM(M, 0.0))
        rows["dlnsig"].append(cos.dlnsig_dlnM(M))
        rows["dndlnM"].append(np.array([cos.dndlnM(M, z) for z in Z_MF]))
        rows["conc"].append(np.array([[cos.conc(m, z, cos.h) for m in M] for z in Z_MF]))
        rows["Sigma_cr"].append([cos.Sigma_cr(a, b) for a, b in PAIRS])
        print("cosmology", rows["params"][-1], "sigma8(tophat)", cos.sigma_tophat8(), flush=True)
    out = {k: np.array(v, float) for k, v in rows.items()}
    out.update(z=Z, M=M, z_mf=Z_MF, pairs=PAIRS)
    np.savez_compressed(REPO / "tests" / "golden" / "cosmo_ref.npz", **out)


if __name__ == "__main__":
    main()
