"""Learned per-plane log-CF surrogate (BF16 MLP on the tensor cores) and its judge.

The per-plane log-CF of a lens plane at redshift z_l (source z_s = 1) is the compensated
compound-Poisson sum over the plane's (halo mass x impact parameter) cells,
    Lambda_p(k) = sum_c w_c (e^{i k kap_c} - 1 - i k kap_c)
              = L_raw(k) - i k sum_c w_c kap_c,      L_raw(k) = sum_c w_c (e^{i k kap_c} - 1).
The exact solver is the engine's 1-D CF sweep (sgl_sweep_eval, FP64).  The MLP learns the
compensated Lambda_p as a function of (h, Om, sigma8, Ok, w0, wa, z_l, ln k) through the outputs
    t0 = ln |Lambda_p|,   t1 = arg(-Lambda_p)
(Re(-Lambda_p) = sum w (1 - cos k kap) >= 0, so t1 stays in [-pi/2, pi/2] without wrapping: ~0 at
small k, -> pi/2 at large k), so that a fixed absolute error in t is a fixed RELATIVE error in the
log-CF.  (Learning the uncompensated L_raw instead and subtracting the exact i k sum w kap loses
the small-k value to cancellation: its leading term is of second order in k.)  Architecture: 8 -> 6 x 256 SiLU -> 2, BF16 weights and
activations in the GEMMs (tcgen05.mma.kind::f16, FP32 accumulation in TMEM), FP32 master weights,
AdamW, MSE on t.  The judge is a two-member ensemble: a plane is re-evaluated by the exact solver
when the members disagree by more than the threshold in ln CF (1e-5 by default).

Synthetic planes (stand-in for the reference's population build, with the synthetic CF-sweep
microbenchmark's shapes): 256 log-spaced masses 1e8-1e16 Msun/h x 512 log-spaced impact parameters
1e-3-1e2 r_s; kappa = A(z_l, cosmology) (M/1e12)^0.3 F(b; c(M)) with the truncated-NFW projection F
and c = 5 (M/1e12)^-0.1; rates w = R(z_l, cosmology) M^-0.9 exp(-M/M*) dlnM 2 pi b^2 dlnb with
M* = 1e15 (sigma8/0.811)^4.  A follows the lensing efficiency D_l D_ls / D_s and R the comoving
volume per unit redshift of a CPL (w0, wa) cosmology with curvature Ok.
"""
from __future__ import annotations

import math

import numpy as np

from .workloads import nfw_trunc_projected

NM, NB = 256, 512
BOX = np.array([[0.6, 0.8], [0.2, 0.4], [0.7, 0.9], [-0.05, 0.05], [-1.3, -0.7], [-0.5, 0.5]])
ZS = 1.0
LNK = (math.log(1e-2), math.log(1e6))


# ------------------------------------------------------------------ synthetic planes
class PlaneModel:
    """Cells of one lens plane for a cosmology theta = (h, Om, sigma8, Ok, w0, wa)."""

    def __init__(self):
        self.M = np.geomspace(1e8, 1e16, NM)
        self.b = np.geomspace(1e-3, 1e2, NB)
        c = 5.0 * (self.M / 1e12) ** -0.1
        F = nfw_trunc_projected(self.b[None, :], c[:, None])                  # (NM, NB)
        self.kapF = ((self.M / 1e12) ** 0.3)[:, None] * F
        dlnb = math.log(self.b[1] / self.b[0])
        self.dlnM = math.log(self.M[1] / self.M[0])
        self.area = 2 * math.pi * self.b ** 2 * dlnb
        a0, r0 = self._amp(np.array([0.674, 0.315, 0.811, 0.0, -1.0, 0.0]), 0.5)
        self.A0, self.R0 = 0.05 / a0, 3.7e6 / 128 / (r0 * self._rate_sum(0.811))

    @staticmethod
    def _distances(theta, z):
        h, Om, s8, Ok, w0, wa = theta
        zz = np.linspace(0.0, max(ZS, float(np.max(z))), 2001)
        Ode = 1.0 - Om - Ok
        fde = (1 + zz) ** (3 * (1 + w0 + wa)) * np.exp(-3 * wa * zz / (1 + zz))
        E = np.sqrt(Om * (1 + zz) ** 3 + Ok * (1 + zz) ** 2 + Ode * fde)
        chi = np.concatenate([[0.0], np.cumsum(0.5 * (1 / E[1:] + 1 / E[:-1]) * np.diff(zz))])

        def dm(x):
            if Ok > 0:
                return np.sinh(math.sqrt(Ok) * x) / math.sqrt(Ok)
            if Ok < 0:
                return np.sin(math.sqrt(-Ok) * x) / math.sqrt(-Ok)
            return x
        chi_z = np.interp(z, zz, chi)
        E_z = np.interp(z, zz, E)
        return dm(chi_z), dm(np.interp(ZS, zz, chi)), chi_z, E_z

    def _amp(self, theta, zl):
        Dl, Ds, chi, E = self._distances(theta, np.atleast_1d(zl))
        Ok = theta[3]
        Dls = (Ds * np.sqrt(1 + Ok * Dl ** 2) - Dl * math.sqrt(1 + Ok * Ds ** 2)) / (1 + ZS)
        eff = (Dl / (1 + np.atleast_1d(zl))) * Dls / (Ds / (1 + ZS))
        A = eff * math.sqrt(theta[1] / 0.315)
        R = chi ** 2 / E * (theta[1] / 0.315) / 128.0
        return float(A[0]), float(R[0])

    def _rate_sum(self, s8):
        Ms = 1e15 * (s8 / 0.811) ** 4
        return float(np.sum(self.M ** -0.9 * np.exp(-self.M / Ms) * self.dlnM) * np.sum(self.area))

    def cells(self, theta, zl):
        """(kappa, w) of the plane, flattened (NM * NB)."""
        a, r = self._amp(np.asarray(theta, float), zl)
        Ms = 1e15 * (theta[2] / 0.811) ** 4
        nm = self.M ** -0.9 * np.exp(-self.M / Ms) * self.dlnM
        kap = (self.A0 * a) * self.kapF
        w = (self.R0 * r) * nm[:, None] * self.area[None, :]
        return kap.ravel(), w.ravel()


def sample_inputs(n_planes, nk, seed):
    """Latin-hypercube cosmologies and planes (z_l in (0.02, 0.98)) and per-plane ln k in the range."""
    rng = np.random.default_rng(seed)
    u = (rng.permuted(np.tile(np.arange(n_planes), (7, 1)), axis=1).T + rng.random((n_planes, 7))) / n_planes
    theta = BOX[:, 0] + u[:, :6] * (BOX[:, 1] - BOX[:, 0])
    zl = 0.02 + 0.96 * u[:, 6]
    lnk = LNK[0] + (LNK[1] - LNK[0]) * np.sort(rng.random((n_planes, nk)), axis=1)
    return theta, zl, lnk


def solve_planes(engine, model, theta, zl, lnk, precision=0):
    """Exact compensated per-plane log-CF Lambda_p(k) from the engine's CF sweep (FP64 default)."""
    out = np.empty(lnk.shape, complex)
    for p in range(len(zl)):
        kap, w = model.cells(theta[p], zl[p])
        engine.sweep_set_cells(kap, w)
        out[p] = engine.sweep(np.exp(lnk[p]), precision)
    return out


def features(theta, zl, lnk):
    """(n_planes * nk, 8) inputs scaled to [-1, 1]."""
    n, nk = lnk.shape
    X = np.empty((n, nk, 8), np.float32)
    th = 2 * (theta - BOX[:, 0]) / (BOX[:, 1] - BOX[:, 0]) - 1
    X[:, :, :6] = th[:, None, :]
    X[:, :, 6] = (2 * (zl - 0.02) / 0.96 - 1)[:, None]
    X[:, :, 7] = 2 * (lnk - LNK[0]) / (LNK[1] - LNK[0]) - 1
    return X.reshape(n * nk, 8)


def targets(lam):
    """(ln |Lambda|, arg(-Lambda)) of the compensated per-plane log-CF."""
    return np.stack([np.log(np.abs(lam)), np.angle(-lam)], -1).reshape(-1, 2).astype(np.float32)


def untarget(T):
    return -np.exp(T[..., 0] + 1j * T[..., 1])


# ------------------------------------------------------------------ the MLP (tensor-core kernels)
class MLP:
    """8 -> width^depth SiLU -> 2 on the engine's stream; weights are torch tensors (device memory)."""

    def __init__(self, engine, width=256, depth=6, seed=0, n_in=8, n_out=2):
        import torch
        self.torch = torch
        self.eng = engine
        self.dev = torch.device("cuda", engine.device)
        self.stream = torch.cuda.ExternalStream(engine.stream, device=self.dev)
        self.sizes = [n_in] + [width] * depth + [n_out]
        rng = np.random.default_rng(seed)
        with torch.cuda.stream(self.stream):
            self.W, self.b, self.mW, self.vW, self.mb, self.vb = [], [], [], [], [], []
            for a, c in zip(self.sizes[:-1], self.sizes[1:]):
                w = rng.standard_normal((a, c)).astype(np.float32) * math.sqrt(2.0 / a)
                self.W.append(torch.tensor(w, device=self.dev))
                self.b.append(torch.zeros(c, device=self.dev))
                for lst, shape in ((self.mW, (a, c)), (self.vW, (a, c)), (self.mb, (c,)), (self.vb, (c,))):
                    lst.append(torch.zeros(shape, device=self.dev))
        self.step_count = 0

    def _gemm(self, M, N, K, A, ars, acs, B, brs, bcs, C, crs, ccs):
        e = self.eng
        e._check(e._L.sgl_gemm_bf16(e._h, M, N, K, A.data_ptr(), ars, acs, B.data_ptr(), brs, bcs, C.data_ptr(),
                                    crs, ccs, 1.0), "sgl_gemm_bf16")

    def forward(self, X, keep=False):
        """X: (n, 8) float32 device tensor -> (n, 2); keep=True stores activations for backward."""
        torch, e = self.torch, self.eng
        n = X.shape[0]
        acts, pre = [X], []
        with torch.cuda.stream(self.stream):
            A = X
            for l, (W, b) in enumerate(zip(self.W, self.b)):
                a, c = W.shape
                Z = torch.empty((n, c), device=self.dev)
                self._gemm(n, c, a, A, a, 1, W, c, 1, Z, c, 1)
                Zb = torch.empty_like(Z) if keep else Z
                out = torch.empty_like(Z)
                last = l == len(self.W) - 1
                e._check(e._L.sgl_mlp_bias_act(e._h, n, c, Z.data_ptr(), b.data_ptr(), Zb.data_ptr(), out.data_ptr(),
                                               0 if last else 1), "sgl_mlp_bias_act")
                if keep:
                    pre.append(Zb)
                    acts.append(out)
                A = out
        if keep:
            self._acts, self._pre = acts, pre
        return A

    def backward_step(self, dY, lr, wd=1e-4, b1=0.9, b2=0.999, eps=1e-8):
        """Back-propagates dY (d loss / d output) through the stored activations, then one AdamW step."""
        torch, e = self.torch, self.eng
        n = dY.shape[0]
        grads = []
        with torch.cuda.stream(self.stream):
            dA = dY
            for l in range(len(self.W) - 1, -1, -1):
                W = self.W[l]
                a, c = W.shape
                if l == len(self.W) - 1:
                    dZ = dA
                else:
                    dZ = torch.empty_like(dA)
                    e._check(e._L.sgl_mlp_act_grad(e._h, n, c, dA.data_ptr(), self._pre[l].data_ptr(), dZ.data_ptr()),
                             "sgl_mlp_act_grad")
                dW = torch.empty((a, c), device=self.dev)
                Aprev = self._acts[l]
                self._gemm(a, c, n, Aprev, 1, a, dZ, c, 1, dW, c, 1)           # A^T dZ
                db = torch.empty(c, device=self.dev)
                e._check(e._L.sgl_mlp_col_sum(e._h, n, c, dZ.data_ptr(), db.data_ptr()), "sgl_mlp_col_sum")
                grads.append((l, dW, db))
                if l > 0:
                    dA = torch.empty((n, a), device=self.dev)
                    self._gemm(n, a, c, dZ, c, 1, W, 1, c, dA, a, 1)           # dZ W^T
            self.step_count += 1
            for l, dW, db in grads:
                for w, g, m, v in ((self.W[l], dW, self.mW[l], self.vW[l]), (self.b[l], db, self.mb[l], self.vb[l])):
                    e._check(e._L.sgl_mlp_adamw(e._h, w.numel(), w.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(),
                                                lr, b1, b2, eps, wd, self.step_count), "sgl_mlp_adamw")
        return grads

    def loss_grad(self, pred, Y):
        import ctypes as C
        torch, e = self.torch, self.eng
        with torch.cuda.stream(self.stream):
            dY = torch.empty_like(pred)
            loss = C.c_double()
            e._check(e._L.sgl_mlp_mse(e._h, pred.numel(), pred.data_ptr(), Y.data_ptr(), dY.data_ptr(), C.byref(loss)),
                     "sgl_mlp_mse")
        return loss.value, dY

    def train(self, X, Y, epochs=20, batch=16384, lr=2e-3, lr_final=1e-5, seed=0, log=None):
        """X, Y: float32 device tensors.  Cosine learning-rate decay; returns the per-epoch mean loss."""
        torch = self.torch
        n = X.shape[0]
        steps = max(1, n // batch)
        rng = np.random.default_rng(seed)
        hist = []
        total = epochs * steps
        it = 0
        for ep in range(epochs):
            with torch.cuda.stream(self.stream):
                perm = torch.tensor(rng.permutation(n), device=self.dev)
            tot = 0.0
            for s in range(steps):
                lr_t = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / total))
                with torch.cuda.stream(self.stream):
                    idx = perm[s * batch:(s + 1) * batch]
                    xb, yb = X[idx].contiguous(), Y[idx].contiguous()
                pred = self.forward(xb, keep=True)
                loss, dY = self.loss_grad(pred, yb)
                self.backward_step(dY, lr_t)
                tot += loss
                it += 1
            hist.append(tot / steps)
            if log:
                log(f"epoch {ep}: loss {hist[-1]:.3e}")
        return hist

    def predict(self, X, batch=65536, host=False):
        """Outputs for X (device tensor).  host=True returns a NumPy array after the engine's stream
        has finished (torch's own streams are not ordered after the engine's kernels)."""
        torch = self.torch
        outs = []
        for s in range(0, X.shape[0], batch):
            outs.append(self.forward(X[s:s + batch].contiguous()))
        with torch.cuda.stream(self.stream):
            out = torch.cat(outs)
        if host:
            self.stream.synchronize()
            return out.cpu().numpy()
        return out


def reference_grads(W, b, X, Y):
    """FP64 NumPy forward / backward of the same MLP (the CPU oracle of the gradient check): returns
    (loss, [(dW, db)] from the first layer on)."""
    acts, pre = [X.astype(np.float64)], []
    A = acts[0]
    for l, (w, bb) in enumerate(zip(W, b)):
        Z = A @ w.astype(np.float64) + bb.astype(np.float64)
        pre.append(Z)
        A = Z if l == len(W) - 1 else Z / (1 + np.exp(-Z))
        acts.append(A)
    d = A - Y.astype(np.float64)
    loss = float(np.mean(d ** 2))
    dA = 2 * d / d.size
    out = []
    for l in range(len(W) - 1, -1, -1):
        Z = pre[l]
        if l == len(W) - 1:
            dZ = dA
        else:
            s = 1 / (1 + np.exp(-Z))
            dZ = dA * s * (1 + Z * (1 - s))
        out.append((acts[l].T @ dZ, dZ.sum(0)))
        dA = dZ @ W[l].astype(np.float64).T
    return loss, out[::-1]


# ------------------------------------------------------------------ ensemble and judge
def to_device(engine, *arrays):
    import torch
    dev = torch.device("cuda", engine.device)
    with torch.cuda.stream(torch.cuda.ExternalStream(engine.stream, device=dev)):
        return [torch.tensor(np.ascontiguousarray(a), device=dev) for a in arrays]


class Surrogate:
    """Two-member ensemble of MLPs; log-CF prediction, disagreement and the judge."""

    def __init__(self, engine, members=2, width=256, depth=6, seed=0):
        self.eng = engine
        self.mlps = [MLP(engine, width, depth, seed=seed + 17 * i) for i in range(members)]

    def train(self, X, Y, epochs=20, batch=16384, lr=2e-3, log=None):
        Xd, Yd = to_device(self.eng, X, Y)
        return [m.train(Xd, Yd, epochs=epochs, batch=batch, lr=lr, seed=i, log=log) for i, m in enumerate(self.mlps)]

    def predict(self, X):
        """Per-member transformed outputs, (members, n, 2) host arrays."""
        (Xd,) = to_device(self.eng, X)
        return np.stack([m.predict(Xd, host=True) for m in self.mlps])

    def log_cf(self, X):
        """Ensemble-mean per-plane log-CF and the members' disagreement |Lambda_1 - Lambda_2| (the
        judge's error estimate).  X rows are planes x k, flattened."""
        L = untarget(self.predict(X))                            # (members, n)
        disagree = np.abs(L[0] - L[-1]) if len(L) > 1 else np.zeros(L.shape[1])
        return L.mean(0), disagree


def judge(engine, model, sur, theta, zl, lnk, threshold=1e-5):
    """Surrogate log-CF for every plane; planes whose ensemble disagreement exceeds `threshold` in
    ln CF at any k are re-evaluated by the exact FP64 solver.  Returns (Lambda, fallback mask)."""
    n, nk = lnk.shape
    lam, dis = sur.log_cf(features(theta, zl, lnk))
    lam = lam.astype(complex).reshape(n, nk)
    bad = dis.reshape(n, nk).max(1) > threshold
    if bad.any():
        idx = np.nonzero(bad)[0]
        lam[idx] = solve_planes(engine, model, theta[idx], zl[idx], lnk[idx])
    return lam, bad


# ------------------------------------------------------------------ surrogate + judge PDF sweep
def instance_planes(theta, n_planes=64):
    """Lens planes of one z_s = 1 instance: midpoints of n_planes equal slices of (0, 1)."""
    zl = (np.arange(n_planes) + 0.5) / n_planes
    return np.repeat(np.asarray(theta, float)[None, :], n_planes, 0), zl


def kappa_pdf_from_logcf(lam_tot, k, lnmu):
    """FP64 inversion of a 1-D kappa CF exp(lam_tot(k)) on a uniform k grid (k[0] = 0, trapezoid) to
    dP/dln mu at lnmu, with mu = (1 - kappa)^-2:  P(kappa) = (1/pi) int_0^K Re[e^{lam - i k kappa}] dk,
    dP/dln mu = P(kappa) (1 - kappa) / 2."""
    kap = 1.0 - np.exp(-0.5 * lnmu)
    wk = np.full(k.size, k[1] - k[0])
    wk[0] *= 0.5
    wk[-1] *= 0.5
    cf = np.exp(lam_tot) * wk
    P = (np.cos(np.outer(kap, k)) @ cf.real + np.sin(np.outer(kap, k)) @ cf.imag) / np.pi
    return P * (1.0 - kap) / 2.0


def pdf_sweep(engine, model, sur, thetas, n_planes=64, nk=2048, kmax=2000.0, lnmu=None, threshold=1e-5):
    """Surrogate + judge PDFs for instances (cosmologies at z_s = 1) and the plain-solver PDFs.
    Returns dict with both PDF sets, per-instance fallback fractions and the wall times."""
    import time
    if lnmu is None:
        lnmu = np.linspace(-0.5, 2.0, 4096)
    k = np.linspace(0.0, kmax, nk)
    lnk = np.log(np.maximum(k[1:], 1e-300))
    out = {"P_sur": [], "P_plain": [], "fallback": [], "t_sur": 0.0, "t_plain": 0.0}
    for th in thetas:
        T, zl = instance_planes(th, n_planes)
        L = np.tile(lnk, (n_planes, 1))
        t0 = time.perf_counter()
        lam, bad = judge(engine, model, sur, T, zl, L, threshold=threshold)
        tot = np.concatenate([[0.0], lam.sum(0)])
        out["P_sur"].append(kappa_pdf_from_logcf(tot, k, lnmu))
        t1 = time.perf_counter()
        exact = solve_planes(engine, model, T, zl, L)
        tot_x = np.concatenate([[0.0], exact.sum(0)])
        out["P_plain"].append(kappa_pdf_from_logcf(tot_x, k, lnmu))
        t2 = time.perf_counter()
        out["t_sur"] += t1 - t0
        out["t_plain"] += t2 - t1
        out["fallback"].append(float(bad.mean()))
    out["lnmu"] = lnmu
    return out
