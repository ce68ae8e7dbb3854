"""FP64 CPU oracle for the characteristic exponent ln Phi(k_kappa, k_gamma).

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA path is compared with;
the product package never imports it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may use it.

It restates, in plain NumPy/SciPy, the algorithm of the reference package
(sgl_analytic v0.2.0, ``src/sgl_analytic/sgl_full.py``):

* ``sep_gamma_nodes``   <- ``_sep_gamma_nodes``       sgl_full.py:2631-2661
* ``sep_rows``          <- ``_sep_lam_kernel``        sgl_full.py:2586-2619
* ``cheb_lobatto``      <- ``_cheb_lobatto_matrix``   sgl_full.py:2665-2680
* ``j0m1``              <- ``_j0m1``                  sgl_full.py:2576-2582
* ``psi1_direct``       <- ``_lam_worker_block``      sgl_full.py:2682-2704
* ``OracleLam.psi1_sep``<- ``Lam._sep_raw``           sgl_full.py:3040-3086
* ``XiGroups``          <- ``Lam.__init__`` xi part   sgl_full.py:2799-2861
* ``OracleLam.qxi``     <- ``Lam._Qxi_gauss``         sgl_full.py:2869-2951
* ``OracleLam.q_interp``<- ``Lam._Q_interpolated``    sgl_full.py:2953-3022 (unblocked path)
* ``OracleLam.__call__``<- ``Lam._direct_call``       sgl_full.py:3088-3131 (C=None, no exact-S)
* ``OracleLam.sigma``   <- ``Lam.sigma``              sgl_full.py:3437-3452

Parity is pinned by ``tests/test_oracle_golden.py`` against the reference's stored golden PDF
``tests/reference/pdf_zs1.json`` (copied into ``tests/golden/``) and against values computed by
the reference's own code on the same cells (``tests/golden/make_fixtures.py``).
"""
from __future__ import annotations

import numpy as np
import scipy.special as sp

# separable-evaluation constants, sgl_full.py:3036-3038
SEP_THETA, SEP_MG, SEP_SMAX = 0.5, 8, 64
SEP_MIN_POINTS = 200_000
XI_PRUNE = 1e-7            # Lam(xi_prune=1e-7), sgl_full.py:2733
XI_COARSE = 101            # Lam(xi_coarse=101)
KG_BLOCK = 512             # Lam.KG_BLOCK, sgl_full.py:3030


def centers_signed(e):
    """Signed-log bin centres (sgl_full.py:466-468): geometric mean, 0 for the bin across 0."""
    return np.where(e[:-1] * e[1:] > 0, np.sign(e[1:]) * np.sqrt(np.abs(e[:-1] * e[1:])), 0.0)


def j0m1(x):
    """J0(x) - 1 with the small-argument series below 1e-3 (sgl_full.py:2576-2582)."""
    x = np.asarray(x, float)
    out = sp.j0(x) - 1.0
    s = x < 1e-3
    out[s] = -x[s] ** 2 / 4 * (1 - x[s] ** 2 / 16)
    return out


def psi1_direct(k0, g0, w, kk, kg, kg_block=KG_BLOCK):
    """Dense direct sum_c w_c (e^{i kk kap_c} J0(kg gam_c) - 1 - i kk kap_c), split into
    O(A)/O(B) pieces exactly as _lam_worker_block (sgl_full.py:2682-2704)."""
    kk = np.asarray(kk, float)
    kg = np.asarray(kg, float)
    out = np.empty((kk.size, kg.size), complex)
    for a in range(0, kg.size, kg_block):
        b = min(a + kg_block, kg.size)
        x = np.outer(g0, kg[a:b])
        J = sp.j0(x)
        B = J - 1.0
        s = x < 1e-3
        if np.any(s):
            B[s] = -x[s] ** 2 / 4 * (1 - x[s] ** 2 / 16)
        base = w @ B
        for lo in range(0, kk.size, 64):
            hi = min(lo + 64, kk.size)
            ph = np.outer(kk[lo:hi], k0)
            re = ((np.cos(ph) - 1) * w) @ J
            im = ((np.sin(ph) - ph) * w) @ J + (ph * w) @ B
            out[lo:hi, a:b] = re + 1j * im + base[None, :]
    return out


def sep_gamma_nodes(g0, w, ig, eg, kg_max, theta=SEP_THETA, mg=SEP_MG, smax=SEP_SMAX):
    """Chebyshev sub-bin gamma nodes + Lagrange weights (sgl_full.py:2631-2661).

    Each occupied fine gamma bin [lo, hi) is cut into ns = ceil(kg_max (hi-lo) / (2 theta))
    equal sub-bins; a cell's weight is spread over the mg Chebyshev nodes of its sub-bin with
    the Lagrange basis evaluated at its centroid.  Bins needing more than smax sub-bins are
    flagged ``direct``.  Returns (nodes (N*mg,), wl (Nc, mg), cols (Nc, mg), direct (Nc,))."""
    lo, hi = eg[ig], eg[ig + 1]
    ns = np.maximum(1, np.ceil(kg_max * (hi - lo) / (2 * theta))).astype(np.int64)
    direct = ns > smax
    sep = ~direct
    j = np.minimum(((g0 - lo) / (hi - lo) * ns).astype(np.int64), ns - 1)
    sl = lo + j * (hi - lo) / ns
    sh = lo + (j + 1) * (hi - lo) / ns
    t = np.cos((2 * np.arange(mg) + 1) * np.pi / (2 * mg))[::-1]
    ub, inv = np.unique(np.round(sl[sep], 14), return_inverse=True)
    lo_s, hi_s = sl[sep], sh[sep]
    nodes = np.empty((ub.size, mg))
    nodes[inv] = 0.5 * (lo_s + hi_s)[:, None] + 0.5 * (hi_s - lo_s)[:, None] * t[None, :]
    u = (2 * g0[sep] - lo_s - hi_s) / (hi_s - lo_s)
    L = np.ones((u.size, mg))
    for a in range(mg):
        for b in range(mg):
            if a != b:
                L[:, a] *= (u - t[b]) / (t[a] - t[b])
    wl = np.zeros((g0.size, mg))
    cols = -np.ones((g0.size, mg), np.int64)
    wl[sep] = w[sep, None] * L
    cols[sep] = inv[:, None] * mg + np.arange(mg)
    return nodes.ravel(), wl, cols, direct


def sep_rows(kk, k0, w, wl, cols, n_nodes, chunk=32):
    """Per k_kappa row n (sgl_full.py:2586-2619):
      A1[n]   = sum_c w_c (e^{i k_n kap_c} - 1 - i k_n kap_c)  (cos-1 = -2 sin^2(ph/2);
                sin(ph) - ph by its 3-term series below |ph| = 1e-2)
      T[n, q] = sum_c wl[c, j] e^{i k_n kap_c},  q = cols[c, j].
    The scatter onto gamma nodes is written as a product with the sparse (cells x nodes)
    Lagrange-weight matrix: the same finite sums, summed in a different order."""
    import scipy.sparse as sps
    kk = np.asarray(kk, float)
    nk = kk.size
    Tr = np.zeros((nk, n_nodes))
    Ti = np.zeros((nk, n_nodes))
    A1 = np.zeros(nk, complex)
    sel = np.flatnonzero(cols[:, 0] >= 0)
    mg = cols.shape[1]
    WL = sps.csr_matrix((wl[sel].ravel(), cols[sel].ravel(), np.arange(0, sel.size * mg + 1, mg)),
                        shape=(sel.size, n_nodes))
    WLt = WL.T.tocsr()
    k_sel = k0[sel]
    for lo in range(0, nk, chunk):
        hi = min(lo + chunk, nk)
        ph = np.outer(kk[lo:hi], k0)
        sn = np.sin(ph)
        hs = np.sin(0.5 * ph)
        cm1 = -2.0 * hs * hs
        p2 = ph * ph
        smp = np.where(np.abs(ph) < 1e-2, -ph * p2 / 6.0 * (1.0 - p2 / 20.0 * (1.0 - p2 / 42.0)),
                       sn - ph)
        A1[lo:hi] = (cm1 @ w) + 1j * (smp @ w)
        cr = (cm1 + 1.0)[:, sel]
        Tr[lo:hi] = (WLt @ cr.T).T
        Ti[lo:hi] = (WLt @ sn[:, sel].T).T
    return A1, Tr, Ti


def cheb_lobatto(K, N, x):
    """Chebyshev-Lobatto points on [0, K] and the barycentric interpolation matrix onto x
    (sgl_full.py:2665-2680)."""
    j = np.arange(N)
    t = 0.5 * K * (1.0 - np.cos(j * np.pi / (N - 1)))
    wb = (-1.0) ** j
    wb[0] *= 0.5
    wb[-1] *= 0.5
    d = x[:, None] - t[None, :]
    exact = np.abs(d) <= 1e-14 * K
    L = wb[None, :] / np.where(exact, 1.0, d)
    L /= L.sum(axis=1, keepdims=True)
    hit = exact.any(axis=1)
    L[hit] = exact[hit].astype(float)
    return t, L


class XiGroups:
    """The xi_lin two-point groups as Lam prepares them (sgl_full.py:2799-2861)."""

    def __init__(self, groups, ce_k, ce_g, prune=XI_PRUNE):
        self.kmc = centers_signed(ce_k)
        self.gmc = np.sqrt(ce_g[:-1] * ce_g[1:])
        ngc = ce_g.size - 1
        if prune:
            s0 = max(float(np.max(np.linalg.norm(g["rows"], axis=1))) for g in groups)
            kept = []
            for g in groups:
                k = np.linalg.norm(g["rows"], axis=1) > prune * s0
                if k.any():
                    kept.append({**g, "rows": g["rows"][k]})
            groups = kept
        self.groups = []
        W0, R0, S0 = [], [], []
        U = {0: [], 1: [], 2: []}
        UR = {0: [], 1: [], 2: []}
        US = {0: [], 1: [], 2: []}
        for g in groups:
            p_all, q_all = g["idx"] // ngc, g["idx"] % ngc
            up, pinv = np.unique(p_all, return_inverse=True)
            uq, qinv = np.unique(q_all, return_inverse=True)
            m = int(g["m"])
            rows = g["rows"][:, :-1]
            res = g["rows"][:, -1]
            srow = rows.sum(axis=1)
            self.groups.append(dict(m=m, sign=1.0 if m == 0 else 2.0 * (-1) ** m,
                                    idx_p=up, idx_q=uq, pinv=pinv, qinv=qinv,
                                    rows=rows, res=res, sum_rows=srow, kc=self.kmc[p_all]))
            r = rows.shape[0]
            if m == 0:
                Wg = np.zeros((r, self.kmc.size))
                np.add.at(Wg.T, p_all, rows.T)
                W0.append(Wg); R0.append(res); S0.append(srow)
            if m in U:
                Ug = np.zeros((r, self.gmc.size))
                np.add.at(Ug.T, q_all, rows.T)
                U[m].append(Ug); UR[m].append(res); US[m].append(srow)
        self.W0 = np.vstack(W0) if W0 else None
        self.res0 = np.concatenate(R0) if R0 else None
        self.sum0 = np.concatenate(S0) if S0 else None
        self.stack_g = {m: dict(U=np.vstack(U[m]), res=np.concatenate(UR[m]),
                                sum=np.concatenate(US[m]), sign=1.0 if m == 0 else 2.0 * (-1) ** m)
                        for m in (0, 1, 2) if U[m]}


def groups_from_npz(d, select=None):
    """Rebuild the reference's raw xi group dicts from the flat arrays of a fixture."""
    m, ni, nr = d["xg_m"], d["xg_nidx"], d["xg_nrow"]
    all_idx, all_rows = d["xg_idx"], d["xg_rows"]      # read once (npz members are lazy)
    idx_off = np.concatenate([[0], np.cumsum(ni)])
    row_off = np.concatenate([[0], np.cumsum(nr * (ni + 1))])
    out = []
    for g in range(m.size) if select is None else select:
        idx = np.asarray(all_idx[idx_off[g]:idx_off[g + 1]], np.int64)
        rows = np.asarray(all_rows[row_off[g]:row_off[g + 1]]).reshape(nr[g], ni[g] + 1)
        out.append(dict(m=int(m[g]), idx=idx, rows=rows))
    return out


class OracleLam:
    """ln Phi for a built population: Psi_1 (Poisson) - 1/2 k^2 V + Psi_2 (gauss xi_lin).

    Mirrors Lam for the default chain (C=None, nord=1, no exact-S, lss_var=0, xi=True,
    lam_coarse=0) of sgl_full.py:2711-3452.  ``method`` = "sep" (default; the reference's
    separable evaluation) or "direct" (the dense sum, the reference's lam_method="direct")."""

    def __init__(self, w0, k0, g0, ig, fe_g, V=0.0, xi=None, method="sep", xi_coarse=XI_COARSE):
        self.w0, self.k0, self.g0 = (np.asarray(a, float) for a in (w0, k0, g0))
        self.ig = np.asarray(ig, np.int64)
        self.fe_g = np.asarray(fe_g, float)
        self.V = float(V)
        self.xi = xi
        self.method = method
        self.xi_coarse = xi_coarse
        self._sep_cache = {}

    # ---------------------------------------------------------------- Psi_1
    def psi1_sep(self, kk, kg):
        """Lam._sep_raw (sgl_full.py:3040-3086), including the Chebyshev k_gamma factor and the
        direct tail for cells whose bin needs more than SEP_SMAX sub-bins."""
        key = float(kg[-1])
        st = self._sep_cache.get(key)
        if st is None:
            st = sep_gamma_nodes(self.g0, self.w0, self.ig, self.fe_g, key)
            self._sep_cache = {key: st}
        nodes, wl, cols, direct = st
        A1, Tr, Ti = sep_rows(kk, self.k0, self.w0, wl, cols, nodes.size)
        Kg = float(kg[-1]) if kg.size else 0.0
        Nch = int(0.65 * float(nodes.max()) * Kg + 50) if (nodes.size and Kg > 0) else 0
        if kg.size > 1 and 0 < Nch < 0.6 * kg.size and kg[0] >= 0.0:
            tch, Lch = cheb_lobatto(Kg, Nch, kg)
            Bc = j0m1(np.outer(nodes, tch))
            out = (Tr @ Bc) @ Lch.T + 1j * ((Ti @ Bc) @ Lch.T)
        else:
            Bn = j0m1(np.outer(nodes, kg))
            out = Tr @ Bn + 1j * (Ti @ Bn)
        out += A1[:, None]
        if direct.any():
            e = np.exp(1j * np.outer(kk, self.k0[direct])) * self.w0[direct]
            out += e @ j0m1(np.outer(self.g0[direct], kg))
        return out

    def psi1(self, kk, kg):
        kk, kg = np.asarray(kk, float), np.asarray(kg, float)
        if self.method == "sep" and kk.size * kg.size >= SEP_MIN_POINTS and kg.size > 1:
            return self.psi1_sep(kk, kg)
        return psi1_direct(self.k0, self.g0, self.w0, kk, kg)

    # ---------------------------------------------------------------- Psi_2
    def qxi(self, kk, kg):
        """Lam._Qxi_gauss (sgl_full.py:2869-2951), with its two 1-D reach fast paths."""
        X = self.xi
        kk, kg = np.asarray(kk, float), np.asarray(kg, float)
        if kg.size == 1 and kg[0] == 0.0 and X.W0 is not None:
            G = np.exp(1j * np.outer(kk, X.kmc)) @ X.W0.T
            G -= X.sum0[None, :]
            G += 1j * kk[:, None] * X.res0[None, :]
            return (0.5 * np.sum(G * G, axis=1))[:, None]
        if kk.size == 1 and kk[0] == 0.0 and X.stack_g:
            out = np.zeros((1, kg.size), complex)
            xg = np.outer(X.gmc, kg)
            J = {0: sp.j0(xg), 1: sp.j1(xg), 2: sp.jv(2, xg)}
            for m, d in X.stack_g.items():
                G = d["U"] @ J[m]
                if m == 0:
                    G -= d["sum"][:, None]
                elif m == 1:
                    G += 0.5 * kg[None, :] * d["res"][:, None]
                out[0, :] += 0.5 * d["sign"] * np.sum(G * G, axis=0)
            return out
        ph = np.outer(kk, X.kmc)
        E = np.concatenate([np.cos(ph), np.sin(ph)], axis=0)
        xg = np.outer(X.gmc, kg)
        J = {0: sp.j0(xg), 1: sp.j1(xg), 2: sp.jv(2, xg)}
        out = np.zeros((kk.size, kg.size), complex)
        for g in X.groups:
            r, m = g["rows"].shape[0], g["m"]
            nP, nQ = g["idx_p"].size, g["idx_q"].size
            Hd = np.zeros((r, nP, nQ))
            Hd[:, g["pinv"], g["qinv"]] = g["rows"]
            T = (Hd.reshape(r * nP, nQ) @ J[m][g["idx_q"], :]).reshape(r, nP, kg.size)
            T2 = np.ascontiguousarray(T.transpose(1, 0, 2)).reshape(nP, r * kg.size)
            G = (E[:, g["idx_p"]] @ T2).reshape(2, kk.size, r, kg.size)
            Gr = G[0].transpose(1, 0, 2)
            Gi = G[1].transpose(1, 0, 2)
            if m == 0:
                Gr = Gr - g["sum_rows"][:, None, None]
                Gi = Gi + kk[None, :, None] * g["res"][:, None, None]
            elif m == 1:
                Gr = Gr + 0.5 * kg[None, None, :] * g["res"][:, None, None]
            out += (0.5 * g["sign"]) * (np.sum(Gr ** 2 - Gi ** 2, axis=0)
                                        + 2j * np.sum(Gr * Gi, axis=0))
        return out

    def q_interp(self, kk, kg, n=XI_COARSE, nk=None):
        """Lam._Q_interpolated, unblocked tensor-product path (sgl_full.py:2998-3022): Q on the
        coarse grid k = kmax s^2 (s uniform on [0, 1]), not-a-knot cubic spline in s built axis
        by axis, evaluated with B-spline design matrices at s = sqrt(k / kmax)."""
        from scipy.interpolate import BSpline, make_interp_spline
        nk = n if nk is None else int(nk)
        kk_max, kg_max = float(kk[-1]), float(kg[-1])
        s = np.linspace(0.0, 1.0, n)
        s_k = s if nk == n else np.linspace(0.0, 1.0, nk)
        sk = np.sqrt(np.clip(kk / kk_max, 0.0, 1.0))
        sg = np.sqrt(np.clip(kg / kg_max, 0.0, 1.0))
        Qc = self.qxi(kk_max * s_k ** 2, kg_max * s ** 2)
        out = np.empty((kk.size, kg.size), complex)
        for part, name in ((Qc.real, "real"), (Qc.imag, "imag")):
            s0 = make_interp_spline(s_k, part, k=3, axis=0)
            s1 = make_interp_spline(s, s0.c, k=3, axis=1)
            val = BSpline.design_matrix(sk, s0.t, 3) @ (BSpline.design_matrix(sg, s1.t, 3) @ s1.c).T
            setattr(out, name, val)
        return out

    # ---------------------------------------------------------------- composition
    def __call__(self, kk, kg, nproc=1):
        """Lam._direct_call for the default chain (sgl_full.py:3088-3131)."""
        kk, kg = np.asarray(kk, float), np.asarray(kg, float)
        out = self.psi1(kk, kg)
        out -= 0.5 * np.outer(kk ** 2 * self.V, np.ones(kg.size))
        if self.xi is not None:
            n = self.xi_coarse
            if n and kk.size * kg.size > n ** 2 and kk.size > 1 and kg.size > 1 \
                    and kk[-1] > 0 and kg[-1] > 0:
                out += self.q_interp(kk, kg, n=n)
            else:
                out += self.qxi(kk, kg)
        return out

    def sigma(self):
        """Total sigma_kappa (sgl_full.py:3437-3452; no Cox term, lss_var = 0)."""
        v = float(np.sum(self.w0 * self.k0 ** 2)) + self.V
        if self.xi is not None and self.xi.W0 is not None:
            v += float(np.sum((self.xi.W0 @ self.xi.kmc + self.xi.res0) ** 2))
        return float(np.sqrt(v))


def oracle_from_npz(path, method="sep", xi=True, select=None):
    d = np.load(path)
    X = None
    if xi:
        X = XiGroups(groups_from_npz(d, select), d["ce_k"], d["ce_g"])
    return OracleLam(d["w0"], d["k0"], d["g0"], d["ig"], d["fe_g"], float(d["V"]), X, method=method)


def cf_sweep(kk, kap, w, chunk=8):
    """sum_c w_c (e^{i k kap_c} - 1 - i k kap_c) per k, with the cancellation-free forms of
    _sep_lam_kernel's A1 term (sgl_full.py:2596-2617); also returns sum_c w_c (|cos-1| + |sin-ph|),
    the scale of the roundoff of any summation order."""
    kk = np.asarray(kk, float)
    out = np.empty(kk.size, complex)
    mag = np.empty(kk.size)
    for lo in range(0, kk.size, chunk):
        hi = min(lo + chunk, kk.size)
        ph = np.outer(kk[lo:hi], kap)
        hs = np.sin(0.5 * ph)
        cm1 = -2.0 * hs * hs
        p2 = ph * ph
        smp = np.where(np.abs(ph) < 1e-2, -ph * p2 / 6.0 * (1.0 - p2 / 20.0 * (1.0 - p2 / 42.0)), np.sin(ph) - ph)
        out[lo:hi] = cm1 @ w + 1j * (smp @ w)
        mag[lo:hi] = np.abs(cm1) @ w + np.abs(smp) @ w
    return out, mag
