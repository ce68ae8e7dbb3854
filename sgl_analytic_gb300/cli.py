"""Command line: the reference's flags and JSON schema (sgl_analytic cli.py:24-78), GPU hot path.

    python -m sgl_analytic_gb300 --z-s 1 --out pdf.json [--population pop.npz] [--precision mixed]

Writes xi = ln mu on [-1, 1] (1601 points) and P_s there, xi_tail / P_s_tail on (1, 9]
(1600 points, same normalisation), moments, diagnostics and timings.
"""
from __future__ import annotations

import argparse
import json
from pathlib import Path

import numpy as np

from .pipeline import EXTENSIONS, P, clipped_moments, run


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--z-s", "--zs", dest="zs", type=float, required=True, help="source redshift")
    ap.add_argument("--h", type=float, default=P["h"])
    ap.add_argument("--Om", type=float, default=P["Om"])
    ap.add_argument("--sigma8", "--s8", dest="s8", type=float, default=P["s8"])
    for name in ("Ob", "ns", "zeq"):
        ap.add_argument(f"--{name}", type=float, default=P[name])
    ap.add_argument("--Ok", "--Omega-K", "--Omega_K", dest="Ok", type=float, default=EXTENSIONS["Ok"])
    ap.add_argument("--w0", type=float, default=EXTENSIONS["w0"])
    ap.add_argument("--wa", type=float, default=EXTENSIONS["wa"])
    ap.add_argument("--growth-mode", "--growth_mode", dest="growth_mode", choices=("auto", "ode", "legacy"),
                    default=EXTENSIONS["growth_mode"])
    ap.add_argument("--radiation", choices=("engine", "none"), default=EXTENSIONS["radiation"])
    ap.add_argument("--closure", choices=("gauss", "vp"), default="gauss")
    ap.add_argument("--config", default="full")
    ap.add_argument("--nproc", type=int, default=1, help="processes for the population build")
    ap.add_argument("--out", default=None, help="output JSON (default output/pdf_zs<zs>.json)")
    ap.add_argument("--population", default=None, help="pre-built population .npz (skips the CPU build)")
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="fp64")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    try:
        out, _ = run(a.zs, a.config, nproc=a.nproc,
                     cosmo=dict(h=a.h, Om=a.Om, s8=a.s8, Ob=a.Ob, ns=a.ns, zeq=a.zeq, Ok=a.Ok, w0=a.w0, wa=a.wa,
                                growth_mode=a.growth_mode, radiation=a.radiation),
                     xi_closure=a.closure, xi_out=np.linspace(-1.0, 1.0, 1601), xi_tail=np.linspace(1.005, 9.0, 1600),
                     population=a.population, precision=a.precision, device=a.device)
    except ValueError as exc:
        ap.error(str(exc))
    x = np.array(out["xi"] + out["xi_tail"])
    p = np.array(out["P_s"] + out["P_s_tail"])
    out["moment_interval"] = [out["grid"]["xi_min"], out["grid"]["xi_max"]]
    out["diagnostics"] = dict(grid_mass=float(np.trapezoid(p, x)), negative_mass=float(np.trapezoid(np.maximum(-p, 0), x)),
                              minimum_density=float(p.min()))
    out["clipped"] = clipped_moments(np.array(out["xi"]), np.array(out["P_s"]))
    dest = Path(a.out) if a.out else Path("output") / f"pdf_zs{a.zs:g}.json"
    dest.parent.mkdir(parents=True, exist_ok=True)
    with dest.open("w") as stream:
        json.dump(out, stream, allow_nan=False)
    c = out["clipped"]
    print(f"zs={a.zs:g} sigma_kappa={out['sigma_kappa']:.5f} clipped var={c['var']:.5e} skew={c['skew']:.3f}  "
          f"{out['seconds']:.1f} s -> {dest}")


if __name__ == "__main__":
    main()
