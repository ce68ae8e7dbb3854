"""Workloads with the reference's z_s=1 shapes, built from committed data.

``zs1_population()``: the reference's own z_s=1 default-cosmology population -- all 79,574
occupied fine cells (tests/golden/pop_zs1_sub.npz) -- with 201 xi_lin groups (67 shells x
m = 0, 1, 2, as the reference's z_s=1 build has).  The full groups are 290 MB and are not
committed; each shell's groups are synthesised from the three real groups of shell 30 (their
coarse-cell patterns and rows), scaled to that shell's real Frobenius row norm
(tests/golden/zs1_xi_shell_stats.npz).  Shapes, sizes and cost per PDF are those of the real
problem; the xi values are a deterministic stand-in.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .population import Population

GOLDEN = Path(__file__).resolve().parents[1] / "tests" / "golden"
BASE_SHELL = 30


def zs1_population(golden: Path = GOLDEN) -> Population:
    pop = Population.load(golden / "pop_zs1_sub.npz")
    st = np.load(golden / "zs1_xi_shell_stats.npz")
    norms = st["norms"]
    base = pop.groups()
    m, nrow, nidx, idx, rows = [], [], [], [], []
    for s in range(norms.shape[0]):
        for g in base:
            f = norms[s, g["m"]] / norms[BASE_SHELL, g["m"]]
            m.append(g["m"])
            nrow.append(g["rows"].shape[0])
            nidx.append(g["idx"].size)
            idx.append(g["idx"])
            rows.append((g["rows"] * f).ravel())
    pop.xg_m = np.asarray(m, np.int32)
    pop.xg_nrow = np.asarray(nrow, np.int32)
    pop.xg_nidx = np.asarray(nidx, np.int32)
    pop.xg_idx = np.concatenate(idx).astype(np.int32)
    pop.xg_rows = np.concatenate(rows)
    pop.xg_s0 = float(st["s0"])
    return pop
