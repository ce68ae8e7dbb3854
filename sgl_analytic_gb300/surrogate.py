"""Learned per-plane log-CF surrogate (BF16 MLP on the tensor cores) and its judge.

The surrogate stands in for the source-independent per-plane log-CF H(q; theta, z_l) of the lens planes
of sgl_analytic_gb300.planes (theta = (h, Om, sigma8, Ok, w0, wa)): a plane of thickness dz and lensing
efficiency s adds dz H(s k) to a source's log-CF.  The exact solver is the engine's compensated CF sweep
over the plane's NM x NB cells (sgl_sweep_eval; batched: sgl_cfb_*).  An 8 -> 6 x 256 SiLU -> 2 MLP maps
(h, Om, sigma8, Ok, w0, wa, z_l, ln q), each scaled to [-1, 1] (z_l through ln(1 + z_l)), to the residual
of (ln |H|, arg(-H)) over the plane's two-moment form
    H0(q) = -(mu2 / 2) q^2 / (1 - i q Sbar),   Sbar = mu2 / (2 mu1),
(mu1 = sum w S, mu2 = sum w S^2, in closed form for these planes), which already has the exact small-q
(-mu2 q^2 / 2) and large-q (-i mu1 q) behaviour, so that the network learns an O(1) shape rather than
the 45 units of ln |H| over the q range.  -H lies in the first quadrant, so arg(-H) never wraps.  One
common shift and scale normalise both outputs: a fixed output error is a fixed RELATIVE error of H.
Below q_min = e^LNQ[0] the residual goes to zero as q / q_min (H0 holds the small-q limit).
BF16 weights and activations in the GEMMs (tcgen05.mma.kind::f16, FP32 accumulation in TMEM), FP32
master weights, AdamW, MSE, all on the engine's own kernels.  The judge is a two-member ensemble: the
members' disagreement estimates the error of the mean.
"""
from __future__ import annotations

import math

import numpy as np

from . import planes as P

LNQ = (math.log(1e-4), math.log(4e3))
LZMAX = math.log1p(P.ZMAX)


# ------------------------------------------------------------------ inputs and targets
def features(theta, zl, lnq):
    """(n_planes * nq, 8) float32 inputs scaled to [-1, 1]; theta (n, 6), zl (n,), lnq (n, nq)."""
    theta = np.atleast_2d(theta)
    n, nq = lnq.shape
    X = np.empty((n, nq, 8), np.float32)
    X[:, :, :6] = (2 * (theta - P.BOX[:, 0]) / (P.BOX[:, 1] - P.BOX[:, 0]) - 1)[:, None, :]
    X[:, :, 6] = (2 * np.log1p(zl) / LZMAX - 1)[:, None]
    X[:, :, 7] = 2 * (lnq - LNQ[0]) / (LNQ[1] - LNQ[0]) - 1
    return X.reshape(n * nq, 8)


def baseline(lnq, mu1, mu2):
    """(ln |H0|, arg(-H0)) of the two-moment form at ln q (arrays broadcast)."""
    x = np.exp(lnq) * (mu2 / (2 * mu1))
    return np.log(0.5 * mu2) + 2 * lnq - 0.5 * np.log1p(x * x), np.arctan(x)


def targets(H, lnq, mu1, mu2):
    """Residual (ln |H| - ln |H0|, arg(-H) - arg(-H0)) of the per-plane log-CF, (n, 2) float64; H, lnq
    (planes, nq), mu1 / mu2 per plane."""
    b0, b1 = baseline(lnq, np.asarray(mu1)[:, None], np.asarray(mu2)[:, None])
    return np.stack([(np.log(np.abs(H)) - b0).ravel(), (np.angle(-H) - b1).ravel()], -1)


def untarget(R, lnq, mu1, mu2):
    """H from residuals R (..., planes * nq, 2)."""
    b0, b1 = baseline(lnq, np.asarray(mu1)[:, None], np.asarray(mu2)[:, None])
    return -np.exp(R[..., 0] + b0.ravel() + 1j * (R[..., 1] + b1.ravel()))


def plane_moments(model, theta, zl):
    """(mu1, mu2) of planes (theta[p], zl[p])."""
    bg = P.Background(theta)
    m = np.array([[v[0] for v in model.moments(bg, p, np.array([zl[p]]))] for p in range(len(zl))])
    return m[:, 0], m[:, 1]


# ------------------------------------------------------------------ exact per-plane log-CF
def sample_planes(n, nq, seed):
    """n planes: Latin-hypercube cosmologies, z_l uniform in ln(1 + z_l) on [0, ZMAX], and nq sorted
    ln q per plane, uniform on LNQ."""
    rng = np.random.default_rng(seed)
    u = (np.argsort(rng.random((7, n)), axis=1).T + rng.random((n, 7))) / n
    theta = P.BOX[:, 0] + u[:, :6] * (P.BOX[:, 1] - P.BOX[:, 0])
    zl = np.expm1(u[:, 6] * LZMAX)
    lnq = LNQ[0] + (LNQ[1] - LNQ[0]) * np.sort(rng.random((n, nq)), axis=1)
    return theta, zl, lnq


def solve_planes(engine, model, theta, zl, lnq, precision=0):
    """Exact H(q) of each plane (the engine's CF sweep over its cells; FP64 by default)."""
    bg = P.Background(theta)
    out = np.empty(lnq.shape, complex)
    for p in range(len(zl)):
        S, w = model.cells(bg, p, zl[p])
        engine.sweep_set_cells(S, w)
        out[p] = engine.sweep(np.exp(lnq[p]), precision)
    return out


# ------------------------------------------------------------------ the MLP (tensor-core kernels)
class MLP:
    """8 -> width^depth SiLU -> 2 on the engine's stream; weights are torch tensors (device memory).
    The GEMMs take BF16 weights; split=True feeds each layer's FP32 input as two BF16 parts (hi, lo) so
    that only the weights are rounded to BF16 (twice the tensor-core work of plain BF16 inputs)."""

    def __init__(self, engine, width=256, depth=6, seed=0, n_in=8, n_out=2, split=True):
        import torch
        self.torch = torch
        self.split = split
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
                if self.split:
                    # the layer's input as two BF16 parts [A_hi | A_lo] against [W; W]: the product of the
                    # FP32 input (to 2^-17) with the BF16 weights, FP32 accumulation
                    Ah = A.to(torch.bfloat16).to(torch.float32)
                    A2 = torch.cat([Ah, A - Ah], 1)
                    W2 = torch.cat([W, W], 0)
                    self._gemm(n, c, 2 * a, A2, 2 * a, 1, W2, c, 1, Z, c, 1)
                else:
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

    def train(self, X, Y, steps=2000, batch=16384, lr=2e-3, lr_final=1e-5, seed=0, log=None, log_every=500):
        """X, Y: float32 device tensors.  `steps` AdamW steps on batches drawn uniformly (with
        replacement) on the device, cosine learning-rate decay; returns the loss every log_every steps."""
        torch = self.torch
        n = X.shape[0]
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(int(seed))
        hist, tot, cnt = [], 0.0, 0
        for it in range(steps):
            lr_t = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / max(1, steps)))
            with torch.cuda.stream(self.stream):
                idx = torch.randint(0, n, (batch,), device=self.dev, generator=gen)
                xb, yb = X[idx], Y[idx]
            pred = self.forward(xb, keep=True)
            loss, dY = self.loss_grad(pred, yb)
            self.backward_step(dY, lr_t)
            tot += loss
            cnt += 1
            if cnt == log_every or it == steps - 1:
                hist.append(tot / cnt)
                if log:
                    log(f"step {it + 1}: loss {hist[-1]:.3e}")
                tot, cnt = 0.0, 0
        return hist

    def infer(self, X):
        """Forward pass of the trained network in the engine's fused kernel (sgl_mlp_infer): the same
        arithmetic as forward(), one launch.  X: (n, 8) float32 device tensor -> (n, 2)."""
        import ctypes as C
        torch, e = self.torch, self.eng
        if self.sizes != [8] + [256] * 6 + [2]:
            return self.forward(X)
        with torch.cuda.stream(self.stream):
            Xc = X.contiguous()
            Y = torch.empty((X.shape[0], 2), device=self.dev)
        Wp = (C.c_void_p * 7)(*[w.data_ptr() for w in self.W])
        bp = (C.c_void_p * 7)(*[b.data_ptr() for b in self.b])
        e._check(e._L.sgl_mlp_infer(e._h, int(X.shape[0]), Xc.data_ptr(), 7, Wp, bp, Y.data_ptr()), "sgl_mlp_infer")
        return Y

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



def to_device(engine, *arrays):
    import torch
    dev = torch.device("cuda", engine.device)
    with torch.cuda.stream(torch.cuda.ExternalStream(engine.stream, device=dev)):
        return [torch.tensor(np.ascontiguousarray(a), device=dev) for a in arrays]


# ------------------------------------------------------------------ ensemble
class Surrogate:
    """Two-member ensemble of MLPs with the common target normalisation (shift of t0, one scale)."""

    def __init__(self, engine, members=2, width=256, depth=6, seed=0, split=True):
        self.eng = engine
        self.mlps = [MLP(engine, width, depth, seed=seed + 17 * i, split=split) for i in range(members)]
        self.shift, self.scale = 0.0, 1.0

    def fit_normalisation(self, T):
        self.shift = float(np.mean(T[:, 0]))
        self.scale = float(np.std(T[:, 0]))

    def normalise(self, T):
        return np.stack([(T[:, 0] - self.shift) / self.scale, T[:, 1] / self.scale], -1).astype(np.float32)

    def denormalise(self, Y):
        return np.stack([Y[..., 0] * self.scale + self.shift, Y[..., 1] * self.scale], -1)

    def train(self, X, T, steps=2000, batch=16384, lr=2e-3, log=None, log_every=500):
        """X features, T residual targets; the normalisation is fitted on T.  Returns each member's loss
        history (every log_every steps)."""
        self.fit_normalisation(T)
        Xd, Yd = to_device(self.eng, X, self.normalise(T))
        return [m.train(Xd, Yd, steps=steps, batch=batch, lr=lr, seed=i, log=log, log_every=log_every)
                for i, m in enumerate(self.mlps)]

    def predict(self, X):
        """Per-member (t0, t1), (members, n, 2) host arrays."""
        (Xd,) = to_device(self.eng, X)
        return np.stack([self.denormalise(m.predict(Xd, host=True).astype(np.float64)) for m in self.mlps])

    def log_cf(self, X, lnq, mu1, mu2):
        """Ensemble-mean H and the members' disagreement |H_1 - H_2| at the rows of X (planes x nq, with
        their ln q and plane moments)."""
        H = untarget(self.predict(X), lnq, mu1, mu2)
        dis = np.abs(H[0] - H[-1]) if len(H) > 1 else np.zeros(H.shape[1])
        return H.mean(0), dis


# ------------------------------------------------------------------ production sweep (surrogate + judge)
SWEEP_NQ = 128


def sample_instances(n, seed, zs=None):
    """n Latin-hypercube cosmologies of the box; source redshifts uniform on ZS_RANGE, or all zs."""
    rng = np.random.default_rng(seed)
    u = (np.argsort(rng.random((7, n)), axis=1).T + rng.random((n, 7))) / n
    theta = P.BOX[:, 0] + u[:, :6] * (P.BOX[:, 1] - P.BOX[:, 0])
    z = np.full(n, float(zs)) if zs is not None else P.ZS_RANGE[0] + u[:, 6] * (P.ZS_RANGE[1] - P.ZS_RANGE[0])
    return theta, z


class SweepTables:
    """Planes, k grids and surrogate nodes of a set of instances (theta, z_s): plane p of instance i
    adds dz_p H(s_p k) on k_n = n dk_i, n < nk; its nq nodes span ln q from max(ln(s_p dk_i), LNQ[0])
    to ln(s_p k_max,i)."""

    def __init__(self, model, theta, zs, nk=4096, nq=SWEEP_NQ):
        self.model, self.theta, self.zs, self.nq = model, np.atleast_2d(theta), np.asarray(zs, float), nq
        self.bg = P.Background(self.theta)
        p0, zl, dz, s, inst, dk, sig, m1, m2 = [0], [], [], [], [], [], [], [], []
        for i in range(self.zs.size):
            a, b, c, sg = model.instance(self.bg, i, self.zs[i])
            u, v = model.moments(self.bg, i, a)
            zl.append(a); dz.append(b); s.append(c); m1.append(u); m2.append(v)
            inst.append(np.full(a.size, i))
            p0.append(p0[-1] + a.size)
            sig.append(sg)
            dk.append(P.k_grid(sg, nk)[0])
        self.inst_plane0 = np.array(p0, np.int32)
        self.zl, self.dz, self.s = np.concatenate(zl), np.concatenate(dz), np.concatenate(s)
        self.mu1, self.mu2 = np.concatenate(m1), np.concatenate(m2)
        self.plane_inst = np.concatenate(inst)
        self.sigma, self.dk = np.array(sig), np.array(dk)
        self.nk = np.full(self.zs.size, nk, np.int32)
        kmax = self.dk[self.plane_inst] * (nk - 1)
        with np.errstate(divide="ignore"):
            lo = np.maximum(np.log(self.s * self.dk[self.plane_inst]), LNQ[0])
            top = np.log(self.s * kmax)
        self.lnq0 = lo
        self.hq = np.where(top > lo + 1e-6, (top - lo) / (nq - 1), 1e-3)
        self.q_above_range = int(np.sum(top > LNQ[1] + 1e-9))

    @property
    def n_planes(self):
        return int(self.zl.size)

    def features(self, engine):
        """The ensemble's inputs at every plane's nodes (as surrogate.features), built on the device:
        (planes * nq, 8) float32."""
        import torch
        dev = torch.device("cuda", engine.device)
        with torch.cuda.stream(torch.cuda.ExternalStream(engine.stream, device=dev)):
            th = torch.tensor(2 * (self.theta - P.BOX[:, 0]) / (P.BOX[:, 1] - P.BOX[:, 0]) - 1, device=dev,
                              dtype=torch.float32)
            pi = torch.tensor(self.plane_inst, device=dev)
            zf = torch.tensor(2 * np.log1p(self.zl) / LZMAX - 1, device=dev, dtype=torch.float32)
            l0 = torch.tensor(self.lnq0, device=dev)
            hq = torch.tensor(self.hq, device=dev)
            j = torch.arange(self.nq, device=dev, dtype=torch.float64)
            lnq = l0[:, None] + hq[:, None] * j[None, :]
            qf = (2 * (lnq - LNQ[0]) / (LNQ[1] - LNQ[0]) - 1).to(torch.float32)
            n, nq = self.n_planes, self.nq
            X = torch.empty((n, nq, 8), device=dev, dtype=torch.float32)
            X[:, :, :6] = th[pi][:, None, :]
            X[:, :, 6] = zf[:, None]
            X[:, :, 7] = qf
            return X.reshape(n * nq, 8)

    def plane_cells(self, p):
        """(kappa, w) of plane p for its source: kappa = s S, w = dz w."""
        i = int(self.plane_inst[p])
        S, w = self.model.cells(self.bg, i, self.zl[p])
        return self.s[p] * S, self.dz[p] * w

    def separable(self, planes=None, nk=None, lo=None):
        """sgl_cfb_set_separable arguments for whole instances (planes None), or for single planes on the
        points lo[j] .. lo[j] + nk[j] - 1 of their instance's k grid; V = 0 (the plain compound-Poisson
        log-CF).  Plane p's cells: kappa = s_p a[m] F[m, b], w = dz_p c[m] area[b]."""
        k0 = None
        if planes is None:
            planes = np.arange(self.n_planes)
            p0 = self.inst_plane0
            nk, dk = self.nk, self.dk
        else:
            planes = np.asarray(planes)
            p0 = np.arange(planes.size + 1, dtype=np.int32)
            nk = self.nk[self.plane_inst[planes]] if nk is None else nk
            dk = self.dk[self.plane_inst[planes]]
            k0 = None if lo is None else np.asarray(lo) * dk
        u = np.empty((planes.size, P.NM))
        v = np.empty((planes.size, P.NM))
        inst = self.plane_inst[planes]
        for i in np.unique(inst):
            sel = np.nonzero(inst == i)[0]
            a, c = self.model.factors(self.bg, int(i), self.zl[planes[sel]])
            u[sel] = self.s[planes[sel], None] * a
            v[sel] = self.dz[planes[sel], None] * c
        return dict(F=self.model.F, g=self.model.area, inst_plane0=p0, nk=nk, dk=dk, V=np.zeros(len(nk)), u=u, v=v,
                    k0=k0)


def node_separable(tables, planes, node_lo=None, n_nodes=None):
    """sgl_cfb_set_separable arguments that put each of `planes` on its own nodes' k points, q_j / s_p =
    exp(lnq0_p - ln s_p + j hq_p) (log-spaced: geom), j = node_lo .. node_lo + n_nodes - 1 (all nodes by
    default)."""
    planes = np.asarray(planes)
    lo = np.zeros(planes.size, np.int64) if node_lo is None else np.asarray(node_lo)
    nn = np.full(planes.size, tables.nq) if n_nodes is None else np.asarray(n_nodes)
    d = tables.separable(planes)
    d.update(nk=nn.astype(np.int32), dk=tables.hq[planes],
             k0=tables.lnq0[planes] - np.log(tables.s[planes]) + lo * tables.hq[planes], geom=True)
    return d


def node_band(tables, planes, band, margin=2):
    """Node range [lo, hi) of each plane that covers its k band [first, end) with the interpolation
    stencil and `margin` more nodes on each side."""
    planes = np.asarray(planes)
    inst = tables.plane_inst[planes]
    dk, s = tables.dk[inst], tables.s[planes]
    x = lambda n: (np.log(s * np.maximum(n, 1) * dk) - tables.lnq0[planes]) / tables.hq[planes]
    lo = np.floor(x(band[:, 0])).astype(np.int64) - 1 - margin
    hi = np.ceil(x(band[:, 1] - 1)).astype(np.int64) + 3 + margin
    lo = np.clip(lo, 0, tables.nq - 2)
    hi = np.clip(hi, lo + 2, tables.nq)
    return lo, hi


def plain_node_pdfs(engine, tables, lnmu, precision=1, pdf_precision=0):
    """The plain solver in node form: every plane exact at its nq log-spaced nodes (batched solver), the
    4-point interpolation of the nodes onto the instance's k grid, then the inversion.  Returns (P, ms of
    the node solve)."""
    import time
    import torch
    engine.sur_set(tables.inst_plane0, tables.nk, tables.dk, tables.s, tables.dz, tables.mu1, tables.mu2, tables.lnq0,
                   tables.hq, tables.nq)
    dev = torch.device("cuda", engine.device)
    with torch.cuda.stream(torch.cuda.ExternalStream(engine.stream, device=dev)):
        Y = torch.zeros((1, tables.n_planes * tables.nq, 2), device=dev, dtype=torch.float32)
    engine.cfb_set_separable(**node_separable(tables, np.arange(tables.n_planes)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.cfb_lnphi(precision, host=False)
    ms = 1e3 * (time.perf_counter() - t0)
    engine.sur_nodes_exact(np.arange(tables.n_planes), Y, 1, 0.0, 1.0)
    engine.sur_finish(Y, 1, 0.0, 1.0, np.full(tables.n_planes, -1, np.int32))
    return engine.sur_pdf(lnmu, precision=pdf_precision), ms


def plain_pdfs(engine, tables, lnmu, precision=1):
    """The plain batched solver over every cell of every plane (built on the device from the planes'
    template), then the inversion: (P, device ms of the solve and the inversion)."""
    engine.cfb_set_separable(**tables.separable())
    return engine.cfb_pdf(lnmu, precision=precision, use_graph=False)


def judge_sweep(engine, sur, tables, lnmu, threshold=1e-5, mode="nodes", fallback_precision=1, pdf_precision=0):
    """Surrogate + judge PDFs of the instances of `tables`.  The ensemble runs at every plane's nodes; the
    judge measures, per plane, the members' spread dz |H_1 - H_2| on the instance's k grid and sends work
    back to the plain batched solver (fallback_precision: SGL_MIXED, within 1e-6 of FP64, by default):
      mode "nodes":    every plane whose |Phi|-weighted spread -- the error it can put into Phi -- exceeds
                       `threshold` somewhere, solved exactly at the nodes that cover that band of k (with
                       the interpolation stencil and two more nodes each side), which replace the members'
                       outputs there;
      mode "plane":    every plane whose largest spread exceeds `threshold` (in ln CF), on the whole k grid;
      mode "weighted": every plane whose largest |Phi|-weighted spread exceeds it, on the whole k grid;
      mode "band":     every plane on the band of k from the first to the last point where its
                       |Phi|-weighted spread exceeds it.
    Then the inversion (pdf_precision, FP64 by default).  Returns (P, info): info["fallback_fraction"] is
    the fallback's terms as a fraction of the plain solver's (plane, k) terms (a node counts as nk / nq
    k points), info["planes_fraction"] the fraction of planes sent back."""
    import time
    import torch
    t = {}
    t0 = time.perf_counter()
    engine.sur_set(tables.inst_plane0, tables.nk, tables.dk, tables.s, tables.dz, tables.mu1, tables.mu2, tables.lnq0,
                   tables.hq, tables.nq)
    X = tables.features(engine)
    with torch.cuda.stream(torch.cuda.ExternalStream(engine.stream, device=X.device)):
        Y = torch.stack([m.infer(X) for m in sur.mlps]).contiguous()
    dis, band = engine.sur_judge(Y, len(sur.mlps), sur.shift, sur.scale, threshold)
    t["judge"] = time.perf_counter() - t0
    nk_pl = tables.nk[tables.plane_inst]
    lo = None
    if mode == "plane":
        bad = np.nonzero(dis[:, 0] > threshold)[0]
        nk_bad = nk_pl[bad]
    elif mode == "weighted":
        bad = np.nonzero(dis[:, 1] > threshold)[0]
        nk_bad = nk_pl[bad]
    elif mode == "band":
        bad = np.nonzero(band[:, 1] > 0)[0]
        lo = band[bad, 0].astype(np.int64)
        nk_bad = np.maximum(band[bad, 1] - lo, 2)
        lo = np.minimum(lo, nk_pl[bad] - nk_bad)
    elif mode == "nodes":
        bad = np.nonzero(band[:, 1] > 0)[0]
        node_lo, node_hi = node_band(tables, bad, band[bad])
        nk_bad = node_hi - node_lo
    else:
        raise ValueError(f"unknown judge mode {mode!r}")
    exact = np.full(tables.n_planes, -1, np.int32)
    exact_lo = np.zeros(tables.n_planes, np.int32)
    t1 = time.perf_counter()
    if bad.size and mode == "nodes":
        engine.cfb_set_separable(**node_separable(tables, bad, node_lo, nk_bad))
        engine.cfb_lnphi(fallback_precision, host=False)
        engine.sur_nodes_exact(bad, Y, len(sur.mlps), sur.shift, sur.scale, node_lo)
        nk_bad = nk_bad * (nk_pl[bad] / tables.nq)          # in k-grid terms: a node costs nk / nq points
    elif bad.size:
        engine.cfb_set_separable(**tables.separable(bad, nk_bad, lo))
        engine.cfb_lnphi(fallback_precision, host=False)
        exact[bad] = np.arange(bad.size, dtype=np.int32)
        if lo is not None:
            exact_lo[bad] = lo
    t["fallback"] = time.perf_counter() - t1
    t2 = time.perf_counter()
    engine.sur_finish(Y, len(sur.mlps), sur.shift, sur.scale, exact, exact_lo)
    Pm = engine.sur_pdf(lnmu, precision=pdf_precision)
    t["finish"] = time.perf_counter() - t2
    t["total"] = time.perf_counter() - t0
    frac = float(np.sum(nk_bad)) / float(np.sum(nk_pl)) if bad.size else 0.0
    return Pm, dict(fallback=bad, fallback_nk=nk_bad, fallback_lo=lo, fallback_fraction=frac,
                    planes_fraction=bad.size / tables.n_planes, dis=dis, band=band, times=t)


def pdf_errors(P, Pref, lnmu, tail_from=1.0, tail_floor=1e-9):
    """Per-instance PDF L1 over ln mu and the tail relative error (ln mu > tail_from where the reference
    exceeds tail_floor times its peak)."""
    l1 = np.trapezoid(np.abs(P - Pref), lnmu, axis=-1)
    tail = lnmu > tail_from
    out = []
    for a, b in zip(np.atleast_2d(P), np.atleast_2d(Pref)):
        m = tail & (b > tail_floor * b.max())
        out.append(float(np.max(np.abs(a[m] - b[m]) / b[m])) if m.any() else 0.0)
    return l1, np.array(out)
