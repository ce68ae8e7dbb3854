"""The population build's cell accumulator with its deposits binned on the GPU.

``Cells`` has the interface of the reference's ``Cells`` (sgl_full.py:1282-1533): ``add`` (one object),
``add_weak``, ``xi_begin`` / ``xi_add_shear_tail`` / ``xi_end`` for the xi_lin term, and the attributes
``Lam`` and ``Population.from_cells`` read (``H0``, ``H0k``, ``H0g``, ``Hc``, ``wM``, ``wV``, ``N``,
``dropped``, ``lin``, ``fe``, ``ce``, ``nord``, ``xi``, ``xi_groups``).  The lattices stay in device
memory (sgl_cells_* of the engine); the histograms are read back when an attribute is read.  ``add_many``
deposits a list of objects in one call.

The reference's emitters can deposit into it unchanged: ``install()`` replaces ``sgl_full.Cells`` in an
imported reference module, so ``build_population`` bins on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Engine, _ptr

# the lattices of the default build (sgl_full.py:456-457): (lowest, highest, bins)
FINE = dict(k=(1e-7, 30.0, 480), g=(1e-9, 30.0, 300))
COARSE = dict(k=(1e-7, 30.0, 170), g=(1e-9, 30.0, 110))
G_CLIP = 1.0000001                      # gamma clipped below at this x the fine grid's lowest (sgl_full.py:1324)


def signed_log_edges(spec):
    lo, hi, n = spec
    pos = np.geomspace(lo, hi, n + 1)
    return np.concatenate([-pos[::-1], pos])


def geom_edges(spec):
    lo, hi, n = spec
    return np.geomspace(lo, hi, n + 1)


class Cells:
    """Binned jump cells of one build, split per z-shell, accumulated on the GPU."""

    def __init__(self, nshell, nord, xi=None, fine=None, coarse=None, engine=None, device=0):
        fine = dict(FINE if fine is None else fine)
        coarse = dict(COARSE if coarse is None else coarse)
        self.nord = int(nord)
        self.nshell = int(nshell)
        self.xi = xi
        self.xi_groups = []
        self._fine, self._coarse = fine, coarse
        self.fe = [signed_log_edges(fine["k"]), geom_edges(fine["g"])]
        self.ce = [signed_log_edges(coarse["k"]), geom_edges(coarse["g"])]
        self.engine = engine if engine is not None else Engine(device)
        e = self.engine
        ek, eg, ck, cg = (np.ascontiguousarray(a, np.float64) for a in (*self.fe, *self.ce))
        e._check(e._L.sgl_cells_init(e._h, self.nshell, self.nord, ek.size, _ptr(ek), eg.size, _ptr(eg), ck.size,
                                     _ptr(ck), cg.size, _ptr(cg), G_CLIP * fine["g"][0], float(fine["k"][1])),
                 "sgl_cells_init")
        self._shape_f = (ek.size - 1, eg.size - 1)
        self._shape_c = (self.nshell, self.nord + 1, ck.size - 1, cg.size - 1)
        if xi is not None:
            kp = np.ascontiguousarray(xi["kp"], np.float64)
            c = np.ascontiguousarray(xi["c"], np.float64)
            e._check(e._L.sgl_cells_xi_init(e._h, kp.size, _ptr(kp), _ptr(c), int(xi["mmax"]), int(bool(xi.get("pos")))),
                     "sgl_cells_xi_init")
        self.wM = np.zeros((self.nshell, self.nord + 1))
        self.wV = np.zeros((self.nshell, self.nord + 1))
        self.dropped = 0.0
        self.N = 0.0
        self.lin = {}
        self._node_shell = None
        self._cache = None

    # ---------------------------------------------------------------- deposits
    def add(self, K, G, W, shell, beta, R=None, tang=True, xi_linear=False):
        """One object (Cells.add, sgl_full.py:1314-1385).  Returns None, as the reference's default does."""
        if xi_linear:
            raise NotImplementedError("xi_linear deposits (the SGL_XI_LINEAR_M prototype) are not implemented")
        self.add_many([dict(K=K, G=G, W=W, shell=shell, beta=beta, R=R, tang=tang)])

    def add_many(self, objects):
        """Deposits a list of objects (dicts with K, G, W, shell, beta and, with the xi_lin term, R and
        tang) in order, in one call."""
        if not objects:
            return
        Ks, Gs, Ws, Rs = [], [], [], []
        for ob in objects:
            K = np.asarray(ob["K"], np.float64).ravel()
            G = np.asarray(ob["G"], np.float64).ravel()
            W = np.asarray(ob["W"], np.float64).ravel()
            if not (K.size == G.size == W.size):
                raise ValueError("K, G and W must have one entry per point")
            Ks.append(K)
            Gs.append(G)
            Ws.append(W)
            if self.xi is not None:
                if ob.get("R") is None:
                    raise NotImplementedError(
                        "clustering='xilin' needs each point's lens distance R; this builder path does not supply it")
                R = np.asarray(ob["R"], np.float64).ravel()
                if R.size != K.size:
                    raise ValueError("R must give one lens distance per point")
                Rs.append(R)
        off = np.concatenate([[0], np.cumsum([k.size for k in Ks])]).astype(np.int64)
        K, G, W = (np.ascontiguousarray(np.concatenate(a)) for a in (Ks, Gs, Ws))
        R = np.ascontiguousarray(np.concatenate(Rs)) if Rs else None
        shell = np.array([int(ob["shell"]) for ob in objects], np.int32)
        beta = np.array([float(ob["beta"]) for ob in objects], np.float64)
        tang = np.array([bool(ob.get("tang", True)) for ob in objects], np.uint8)
        sums = np.zeros((len(objects), 3))
        e = self.engine
        e._check(e._L.sgl_cells_add(e._h, len(objects), _ptr(off, C.c_int64), _ptr(K), _ptr(G), _ptr(W),
                                    _ptr(R) if R is not None else None, _ptr(shell, C.c_int32), _ptr(beta),
                                    _ptr(tang, C.c_ubyte), _ptr(sums)), "sgl_cells_add")
        self._cache = None
        for ob, (w_sum, h_sum, lin_sum) in zip(objects, sums):
            self.dropped += w_sum - h_sum
            self.N += w_sum
            key = (int(ob["shell"]), float(ob["beta"]))
            self.lin[key] = self.lin.get(key, 0.0) + lin_sum

    def add_weak(self, m, v, shell, beta):
        """The weak arm's Gaussian moments (Cells.add_weak, sgl_full.py:1525-1533)."""
        if self.xi is not None:
            raise NotImplementedError("clustering='xilin' has no weak (Gaussian) arm")
        key = (shell, float(beta))
        self.lin[key] = self.lin.get(key, 0.0) + m
        for n in range(self.nord + 1):
            self.wM[shell, n] += m * beta**n
            self.wV[shell, n] += v * beta**n

    # ---------------------------------------------------------------- xi_lin nodes
    def xi_begin(self, dchi):
        e = self.engine
        e._check(e._L.sgl_cells_xi_begin(e._h, float(dchi)), "xi_begin")

    def xi_add_shear_tail(self, beta, Gam, Rm, n_area):
        if self.xi is None or self.xi["mmax"] < 1:
            return
        e = self.engine
        e._check(e._L.sgl_cells_xi_shear_tail(e._h, float(beta), float(Gam), float(Rm), float(n_area)),
                 "xi_add_shear_tail")

    def xi_end(self, shell):
        """Closes the node; appends its compressed row groups (dicts shell, m, idx, rows[, W, v0])."""
        e = self.engine
        ng = C.c_int()
        e._check(e._L.sgl_cells_xi_end(e._h, C.byref(ng)), "xi_end")
        nkp = int(np.asarray(self.xi["kp"]).size)
        for g in range(ng.value):
            m, ni, nr = C.c_int32(), C.c_int32(), C.c_int32()
            e._check(e._L.sgl_cells_xi_group(e._h, g, C.byref(m), C.byref(ni), C.byref(nr), None, None, None, None),
                     "xi_group")
            idx = np.zeros(ni.value, np.int32)
            rows = np.zeros((nr.value, ni.value + 1))
            pos = m.value == 0 and bool(self.xi.get("pos"))
            W = np.zeros(ni.value) if pos else None
            v0 = np.zeros(nkp) if pos else None
            e._check(e._L.sgl_cells_xi_group(e._h, g, None, None, None, _ptr(idx, C.c_int32), _ptr(rows),
                                             _ptr(W) if pos else None, _ptr(v0) if pos else None), "xi_group")
            grp = dict(shell=shell, m=m.value, idx=idx.astype(np.int64), rows=rows)
            if pos:
                grp.update(W=W, v0=v0)
            self.xi_groups.append(grp)

    # ---------------------------------------------------------------- lattices
    def _read(self):
        if self._cache is None:
            H0, H0k, H0g = (np.zeros(self._shape_f) for _ in range(3))
            Hc = np.zeros(self._shape_c)
            e = self.engine
            e._check(e._L.sgl_cells_read(e._h, _ptr(H0), _ptr(H0k), _ptr(H0g), _ptr(Hc)), "sgl_cells_read")
            self._cache = (H0, H0k, H0g, Hc)
        return self._cache

    @property
    def H0(self):
        return self._read()[0]

    @property
    def H0k(self):
        return self._read()[1]

    @property
    def H0g(self):
        return self._read()[2]

    @property
    def Hc(self):
        return self._read()[3]


def install(sgl_full_module):
    """Makes an imported reference ``sgl_full`` module build its populations into GPU ``Cells``.
    Returns the class it replaced."""
    old = sgl_full_module.Cells
    sgl_full_module.Cells = Cells
    return old
