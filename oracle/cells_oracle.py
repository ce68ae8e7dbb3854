"""FP64 NumPy oracle of the binned-cell deposit (test infrastructure only; the product never imports it).

Restates the reference's cell accumulator ``Cells`` (sgl_full.py:1282-1533), the step of the population
build into which every emitter (explicit hosts, filaments, subhalo pairs) deposits its points:

  * the lattices: fine and coarse (kappa, gamma) edges, signed-log in kappa (``_edges``,
    sgl_full.py:460-463) and geometric in gamma (sgl_full.py:1293-1294);
  * ``add`` (sgl_full.py:1314-1385): gamma clipped below at 1.0000001 x the fine grid's lower edge;
    each point's fine and coarse bins by searchsorted(side='right') with values on the last edge
    moved into the last bin and out-of-lattice points dropped (``_add_direct_kernel``,
    sgl_full.py:972-1046); per fine bin the sums of w, w kappa, w gamma; per coarse bin and shell the
    sums of w beta^n, n = 0..nord; the object's totals (all w, w inside the fine lattice, and w kappa
    over |kappa| < the fine grid's upper kappa) into ``N``, ``dropped`` and ``lin[(shell, beta)]``;
  * the xi_lin deposit of a lens-redshift node (``xi_begin`` / ``_xi_deposit`` / ``xi_add_shear_tail``
    / ``xi_end``, sgl_full.py:1387-1523, with ``_xi_add_kernel`` 1049-1079, ``_bessel_pack_nb``
    1132-1185 and ``_xi_rate_deposit`` 1270-1279): for every point inside the coarse box, Hx[bin, m, j]
    += beta w J_{2m}(k_j R) (m >= 1 only for tangential shear), the exact first moments
    lx[0, j] += beta w kappa J0(k_j R), lx[1, j] += beta w gamma J2(k_j R), and for the positive
    closure the unweighted rate per coarse bin; at the node's end, per m, the occupied bins' rows plus
    the residual first-moment row, scaled by sqrt(c_j / dchi), compressed through the eigenvectors of
    their Gram matrix to the rows whose singular value exceeds 1e-6 of the largest.

Sums are taken in the reference's order where it is cheap (np.add.at applies repeated indices in
index order, as the reference's sequential loops do), so the histograms agree with the reference
bit for bit; the xi rows follow the per-point kernel's order (the reference's default groups points
of one radius first, a different summation order of the same sums).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.special as sp

FINE = dict(k=(1e-7, 30.0, 480), g=(1e-9, 30.0, 300))          # sgl_full.py:456
COARSE = dict(k=(1e-7, 30.0, 170), g=(1e-9, 30.0, 110))        # sgl_full.py:457
XI_SVD_TOL = 1e-6                                               # sgl_full.py:2436
G_CLIP = 1.0000001                                              # sgl_full.py:1324


def signed_log_edges(spec):
    """sgl_full.py:460-463."""
    lo, hi, n = spec
    pos = np.geomspace(lo, hi, n + 1)
    return np.concatenate([-pos[::-1], pos])


def geom_edges(spec):
    """sgl_full.py:1293-1294."""
    lo, hi, n = spec
    return np.geomspace(lo, hi, n + 1)


def centers(e):
    """Signed geometric bin centres (sgl_full.py:466-468)."""
    return np.where(e[:-1] * e[1:] > 0, np.sign(e[1:]) * np.sqrt(np.abs(e[:-1] * e[1:])), 0.0)


def bin_index(v, e):
    """searchsorted(side='right'), the last edge moved into the last bin: 1..len(e)-1 inside the
    lattice, 0 below, len(e) above or NaN (sgl_full.py:843-862, 1022-1038)."""
    i = np.searchsorted(e, v, side="right")
    i[v == e[-1]] -= 1
    return i


def bessel_even(x, tang):
    """(J0, J2, J4) of x as the deposit evaluates them (sgl_full.py:1132-1185): the power series with
    3 / 6 / 14 terms below x = 0.02 / 0.3 / 2, above it J0, J1 and upward recurrence; J2 = J4 = 0 for
    non-tangential shear."""
    x = np.asarray(x, float)
    J = np.zeros((3,) + x.shape)
    small = x < 2.0
    xs = x[small]
    h = 0.5 * xs
    h2 = h * h
    nt = np.where(xs < 0.02, 3, np.where(xs < 0.3, 6, 14))
    t0 = np.ones_like(xs)
    s0 = np.ones_like(xs)
    t2 = np.full_like(xs, 0.5)
    s2 = t2.copy()
    t4 = np.full_like(xs, 1.0 / 24.0)
    s4 = t4.copy()
    for k in range(1, 14):
        on = k < nt
        f = (-h2) / k
        t0 = np.where(on, t0 * (f / k), t0)
        s0 = np.where(on, s0 + t0, s0)
        t2 = np.where(on, t2 * (f / (k + 2)), t2)
        s2 = np.where(on, s2 + t2, s2)
        t4 = np.where(on, t4 * (f / (k + 4)), t4)
        s4 = np.where(on, s4 + t4, s4)
    J[0][small] = s0
    if tang:
        J[1][small] = s2 * (h * h)
        J[2][small] = s4 * (h * h * h * h)
    xl = x[~small]
    j0, j1 = sp.j0(xl), sp.j1(xl)
    J[0][~small] = j0
    if tang:
        inv = 1.0 / xl
        j2 = 2.0 * inv * j1 - j0
        j3 = 4.0 * inv * j2 - j1
        J[1][~small] = j2
        J[2][~small] = 6.0 * inv * j3 - j2
    return J


def _seq_sum(v):
    """The running sum in index order (the reference's sequential loop; np.cumsum adds in order)."""
    return float(np.cumsum(v)[-1]) if v.size else 0.0


class CellsOracle:
    """The reference's ``Cells`` (sgl_full.py:1282-1533) for one build."""

    def __init__(self, nshell, nord, xi=None, fine=FINE, coarse=COARSE):
        self.nord = nord
        self.xi = xi
        self.xi_groups = []
        self._xi_cur = None
        self.fine, self.coarse = fine, coarse
        self.fe = [signed_log_edges(fine["k"]), geom_edges(fine["g"])]
        self.ce = [signed_log_edges(coarse["k"]), geom_edges(coarse["g"])]
        self.H0 = np.zeros((self.fe[0].size - 1, fine["g"][2]))
        self.H0k = np.zeros_like(self.H0)
        self.H0g = np.zeros_like(self.H0)
        self.Hc = np.zeros((nshell, nord + 1, self.ce[0].size - 1, coarse["g"][2]))
        self.wM = np.zeros((nshell, nord + 1))
        self.wV = np.zeros((nshell, nord + 1))
        self.dropped = 0.0
        self.N = 0.0
        self.lin = {}

    def add(self, K, G, W, shell, beta, R=None, tang=True):
        K, G, W = (np.asarray(a, float).ravel() for a in (K, G, W))
        G = np.clip(G, G_CLIP * self.fine["g"][0], None)
        if self.xi is not None:
            self._xi_deposit(K, G, W, np.asarray(R, float).ravel(), beta, tang)
        nkf, ngf = self.H0.shape
        nkc, ngc = self.Hc.shape[2:]
        a, b = bin_index(K, self.fe[0]), bin_index(G, self.fe[1])
        inf = (a >= 1) & (a <= nkf) & (b >= 1) & (b <= ngf)
        f = (a[inf] - 1) * ngf + (b[inf] - 1)
        np.add.at(self.H0.ravel(), f, W[inf])
        np.add.at(self.H0k.ravel(), f, W[inf] * K[inf])
        np.add.at(self.H0g.ravel(), f, W[inf] * G[inf])
        ac, bc = bin_index(K, self.ce[0]), bin_index(G, self.ce[1])
        inc = (ac >= 1) & (ac <= nkc) & (bc >= 1) & (bc <= ngc)
        c = (ac[inc] - 1) * ngc + (bc[inc] - 1)
        for n in range(self.nord + 1):
            np.add.at(self.Hc[shell, n].ravel(), c, W[inc] * beta**n)
        w_sum = _seq_sum(W)
        h_sum = _seq_sum(W[inf])
        lk = np.abs(K) < self.fine["k"][1]
        lin_sum = _seq_sum(W[lk] * K[lk])
        self.dropped += w_sum - h_sum
        self.N += w_sum
        key = (shell, float(beta))
        self.lin[key] = self.lin.get(key, 0.0) + lin_sum

    def add_weak(self, m, v, shell, beta):
        key = (shell, float(beta))
        self.lin[key] = self.lin.get(key, 0.0) + m
        for n in range(self.nord + 1):
            self.wM[shell, n] += m * beta**n
            self.wV[shell, n] += v * beta**n

    def xi_begin(self, dchi):
        nkc, ngc = self.Hc.shape[2:]
        nkp, mm = self.xi["kp"].size, self.xi["mmax"]
        self._xi_cur = dict(dchi=float(dchi), Hx=np.zeros((nkc, ngc, mm + 1, nkp)), lx=np.zeros((2, nkp)))
        if self.xi.get("pos"):
            self._xi_cur["Wb"] = np.zeros(nkc * ngc)

    def _xi_deposit(self, K, G, W, R, beta, tang):
        cur = self._xi_cur
        nkc, ngc = self.Hc.shape[2:]
        ac, bc = bin_index(K, self.ce[0]), bin_index(G, self.ce[1])
        ok = (ac >= 1) & (ac <= nkc) & (bc >= 1) & (bc <= ngc)
        c = (ac[ok] - 1) * ngc + (bc[ok] - 1)
        if "Wb" in cur:
            np.add.at(cur["Wb"], c, W[ok])
        kp, mm = self.xi["kp"], self.xi["mmax"]
        Hx = cur["Hx"].reshape(nkc * ngc, mm + 1, kp.size)
        bw_all, Ko, Go, Ro = beta * W[ok], K[ok], G[ok], R[ok]
        for a in range(0, c.size, 65536):                    # points in chunks (the J tables are 3 x n x nkp)
            s = slice(a, a + 65536)
            bw = bw_all[s]
            J = bessel_even(np.outer(Ro[s], kp), tang)
            for m in range(mm + 1):
                np.add.at(Hx[:, m, :], c[s], bw[:, None] * J[m])
            cur["lx"][0] += ((bw * Ko[s])[:, None] * J[0]).sum(0)
            if mm >= 1:
                cur["lx"][1] += ((bw * Go[s])[:, None] * J[1]).sum(0)

    def xi_add_shear_tail(self, beta, Gam, Rm, n_area):
        """sgl_full.py:1466-1476."""
        if self._xi_cur is None or self.xi["mmax"] < 1:
            return
        a = self.xi["kp"] * Rm
        self._xi_cur["lx"][1] += beta * n_area * 2 * math.pi * Gam * sp.j1(a) / a

    def xi_end(self, shell):
        """sgl_full.py:1478-1523."""
        cur, self._xi_cur = self._xi_cur, None
        Hx, lx, dchi = cur["Hx"], cur["lx"], cur["dchi"]
        ngc = Hx.shape[1]
        sw = np.sqrt(self.xi["c"] / dchi)
        kmc = centers(self.ce[0])
        gmc = np.sqrt(self.ce[1][:-1] * self.ce[1][1:])
        for m in range(Hx.shape[2]):
            H = Hx[:, :, m, :].reshape(-1, Hx.shape[3])
            idx = np.flatnonzero(np.any(H != 0, axis=1))
            if idx.size == 0:
                if m > 1 or not np.any(lx[m] != 0):
                    continue
                idx = np.array([0])
            Hm = H[idx]
            if m == 0:
                lres = lx[0] - (kmc[idx // ngc][:, None] * Hm).sum(axis=0)
            elif m == 1:
                lres = lx[1] - (gmc[idx % ngc][:, None] * Hm).sum(axis=0)
            else:
                lres = np.zeros(Hm.shape[1])
            A = np.vstack([Hm, lres[None, :]]) * sw[None, :]
            ev, V = np.linalg.eigh(A.T @ A)
            Vd = V[:, ::-1]
            S = np.sqrt(np.maximum(ev[::-1], 0.0))
            keep = S > XI_SVD_TOL * S[0] if S[0] > 0 else np.zeros(S.size, bool)
            if not keep.any():
                continue
            grp = dict(shell=shell, m=m, idx=idx, rows=(A @ Vd[:, keep]).T, S=S[keep])
            if m == 0 and "Wb" in cur:
                grp.update(W=cur["Wb"][idx].copy(), v0=Vd[:, 0].copy())
            self.xi_groups.append(grp)


def quad_form(rows, f):
    """|rows f|^2 for test vectors f (columns): the quantity Psi_2 takes from a group, independent of
    the sign and the rotation of its rows within the kept subspace."""
    return np.sum((rows @ f) ** 2, axis=0)
