"""The binned lens population that the hot path consumes.

A ``Population`` holds exactly what the reference's ``Lam`` reads from a built ``Cells`` object
(sgl_full.py:2759-2861): the occupied fine (kappa, gamma) cells with their weight-averaged
centroids, the fine gamma bin index and edges, the weak-arm variance, and the raw xi_lin groups
with the coarse lattice edges.  It can be taken from a reference ``Cells`` object
(``Population.from_cells``) or read from / written to a compressed ``.npz`` file.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Population:
    w0: np.ndarray
    k0: np.ndarray
    g0: np.ndarray
    ig: np.ndarray
    fe_g: np.ndarray
    V: float = 0.0
    # xi_lin groups, flat: m[g], nrow[g], nidx[g]; idx (sum nidx); rows (sum nrow*(nidx+1))
    xg_m: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    xg_nrow: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    xg_nidx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    xg_idx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    xg_rows: np.ndarray = field(default_factory=lambda: np.zeros(0))
    ce_k: np.ndarray | None = None
    ce_g: np.ndarray | None = None
    xg_s0: float = 0.0          # > 0: largest row norm of the full set (for subsets of groups)
    zs: float | None = None
    # positive (vp) closure built for this population (pos_closure.install): the arrays of
    # Lam.install_vp (u, w, K, ku, gu, cu, cw, gstart, sh_g, ga, gb, gc, glo, ghi, shear_var, eta)
    vp: dict | None = None

    VP_FILE_KEYS = ("u", "w", "K", "ku", "gu", "cu", "cw", "gstart", "sh_g", "ga", "gb", "gc", "glo", "ghi",
                    "shear_var", "eta")

    @property
    def n_cells(self):
        return int(self.w0.size)

    @property
    def has_xi(self):
        return self.xg_m.size > 0 and self.ce_k is not None

    @classmethod
    def from_cells(cls, cells):
        """Cell compaction of Lam.__init__ (sgl_full.py:2759-2775, centroid=True) and the raw
        xi_lin groups (Cells.xi_groups) of a reference ``Cells`` object."""
        H0 = cells.H0
        ik, ig = np.nonzero(H0)
        w0 = H0[ik, ig]
        k0 = cells.H0k[ik, ig] / w0
        g0 = cells.H0g[ik, ig] / w0
        V = float(cells.wV[:, 0].sum())
        gs = list(getattr(cells, "xi_groups", []) or [])
        kw = {}
        if gs:
            kw = dict(xg_m=np.array([int(g["m"]) for g in gs], np.int32),
                      xg_nrow=np.array([g["rows"].shape[0] for g in gs], np.int32),
                      xg_nidx=np.array([g["idx"].size for g in gs], np.int32),
                      xg_idx=np.concatenate([np.asarray(g["idx"]) for g in gs]).astype(np.int32),
                      xg_rows=np.concatenate([np.asarray(g["rows"], float).ravel() for g in gs]),
                      ce_k=np.asarray(cells.ce[0], float), ce_g=np.asarray(cells.ce[1], float))
        return cls(w0=w0, k0=k0, g0=g0, ig=ig.astype(np.int32), fe_g=np.asarray(cells.fe[1], float), V=V, **kw)

    @classmethod
    def load(cls, path, groups=None):
        """Reads a population ``.npz`` (tests/golden format).  groups: optional subset of xi groups."""
        d = np.load(path)
        kw = dict(w0=d["w0"], k0=d["k0"], g0=d["g0"], ig=d["ig"].astype(np.int32), fe_g=d["fe_g"],
                  V=float(d["V"]), zs=float(d["zs"]) if "zs" in d.files else None)
        if "xg_m" in d.files and d["xg_m"].size:
            m, ni, nr = d["xg_m"], d["xg_nidx"].astype(np.int64), d["xg_nrow"].astype(np.int64)
            idx, rows = d["xg_idx"], d["xg_rows"]
            s0 = float(d["xg_s0"]) if "xg_s0" in d.files else 0.0
            if groups is not None:
                io = np.concatenate([[0], np.cumsum(ni)])
                ro = np.concatenate([[0], np.cumsum(nr * (ni + 1))])
                if s0 == 0.0:
                    s0 = max(float(np.max(np.linalg.norm(rows[ro[g]:ro[g + 1]].reshape(nr[g], ni[g] + 1), axis=1)))
                             for g in range(m.size))
                idx = np.concatenate([idx[io[g]:io[g + 1]] for g in groups])
                rows = np.concatenate([rows[ro[g]:ro[g + 1]] for g in groups])
                m, ni, nr = m[groups], ni[groups], nr[groups]
            kw.update(xg_m=np.asarray(m, np.int32), xg_nrow=np.asarray(nr, np.int32),
                      xg_nidx=np.asarray(ni, np.int32), xg_idx=np.asarray(idx, np.int32),
                      xg_rows=np.asarray(rows, float), ce_k=d["ce_k"], ce_g=d["ce_g"], xg_s0=s0)
        if "vp_u" in d.files:
            kw["vp"] = {k: d["vp_" + k] for k in cls.VP_FILE_KEYS if "vp_" + k in d.files}
        return cls(**kw)

    def save(self, path):
        out = dict(w0=self.w0, k0=self.k0, g0=self.g0, ig=self.ig, fe_g=self.fe_g, V=np.float64(self.V),
                   xg_m=self.xg_m, xg_nrow=self.xg_nrow, xg_nidx=self.xg_nidx, xg_idx=self.xg_idx,
                   xg_rows=self.xg_rows, xg_s0=np.float64(self.xg_s0))
        if self.ce_k is not None:
            out.update(ce_k=self.ce_k, ce_g=self.ce_g)
        if self.zs is not None:
            out["zs"] = np.float64(self.zs)
        if self.vp is not None:
            out.update({"vp_" + k: np.asarray(v) for k, v in self.vp.items() if k in self.VP_FILE_KEYS})
        np.savez_compressed(path, **out)

    def groups(self):
        """The xi groups as the reference's dicts (m, idx, rows)."""
        out = []
        io = ro = 0
        for g in range(self.xg_m.size):
            ni, nr = int(self.xg_nidx[g]), int(self.xg_nrow[g])
            out.append(dict(m=int(self.xg_m[g]), idx=self.xg_idx[io:io + ni].astype(np.int64),
                            rows=self.xg_rows[ro:ro + nr * (ni + 1)].reshape(nr, ni + 1)))
            io += ni
            ro += nr * (ni + 1)
        return out
