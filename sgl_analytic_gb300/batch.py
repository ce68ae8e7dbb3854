"""Batched plain solver: many independent PDFs in flight on one GPU.

A thin layer over the engine's native batch (``sgl_batch_*``): ``slots`` contexts on one device,
each with its own CUDA streams and device arena and one resident population, and one native host
thread per slot that runs that slot's PDFs in order.  A PDF is independent of every other PDF, so
the slots exchange nothing; running several at once fills the device's gaps between one PDF's
kernels and the host-side steps of its inversion (grid plan, moments).
"""
from __future__ import annotations

import numpy as np

from ._lib import PRECISIONS, Batch
from .lam import Lam


class BatchSolver:
    """slots: number of contexts (streams) kept busy at once."""

    def __init__(self, slots=4, device=0, precision="mixed"):
        if slots < 1:
            raise ValueError("slots must be >= 1")
        self.slots = int(slots)
        self.precision = precision
        self.batch = Batch(self.slots, device)
        self.engines = self.batch.engines
        self.lams = [None] * self.slots

    def load(self, populations, xi=True):
        """Makes populations resident, one per slot (len(populations) <= slots)."""
        if len(populations) > self.slots:
            raise ValueError("more populations than slots")
        for i, p in enumerate(populations):
            self.lams[i] = Lam(p, xi=xi, engine=self.engines[i], precision=self.precision)
        return self

    @property
    def streams(self):
        return [e.stream for e in self.engines]

    def solve(self, xi_out, repeats=1, keep_all=False, tail_box=True, phi_tol=1e-8, n_xi_wide=500, n_k_int=2400,
              window=False):
        """Runs `repeats` PDFs on every loaded slot, the slots concurrently; returns the last
        (xi, P, meta) of each slot, or with keep_all every slot's list of all its PDFs' P."""
        xi_out = np.asarray(xi_out, float)
        live = [i for i in range(self.slots) if self.lams[i] is not None]
        if not live:
            raise RuntimeError("no population loaded")
        jobs = np.array([i for _ in range(repeats) for i in live], np.int32)
        P, metas = self.batch.pdf(jobs, xi_out, precision=PRECISIONS[self.precision] if isinstance(self.precision, str)
                                  else int(self.precision), tail_box=tail_box, phi_tol=phi_tol, n_xi_wide=n_xi_wide,
                                  n_k_int=n_k_int, window=window)
        out = []
        for i in live:
            rows = np.nonzero(jobs == i)[0]
            if keep_all:
                out.append([P[r] for r in rows])
            else:
                out.append((xi_out, P[rows[-1]], metas[rows[-1]]))
        return out

    def close(self):
        self.batch.close()
