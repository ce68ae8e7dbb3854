"""GPU checks of the learned per-plane log-CF surrogate: BF16 tensor-core GEMMs, back-propagation
against the FP64 NumPy oracle of the same network, training, and the judge's fallback."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from sgl_analytic_gb300._lib import Engine
    return Engine(0)


def test_bf16_gemm_matches_float64(eng):
    """sgl_gemm_bf16 = the BF16-rounded operands' product (FP32 accumulation), any strides."""
    import torch
    from sgl_analytic_gb300.surrogate import to_device
    rng = np.random.default_rng(0)
    for (M, N, K) in [(300, 256, 70), (5, 2, 256), (1000, 130, 33)]:
        A = rng.standard_normal((M, K)).astype(np.float32)
        B = rng.standard_normal((K, N)).astype(np.float32)
        Ad, Bd = to_device(eng, A, B)
        Cd, = to_device(eng, np.zeros((N, M), np.float32))     # write C transposed
        eng._check(eng._L.sgl_gemm_bf16(eng._h, M, N, K, Ad.data_ptr(), K, 1, Bd.data_ptr(), N, 1, Cd.data_ptr(),
                                        1, M, 1.0), "gemm")
        torch.cuda.ExternalStream(eng.stream).synchronize()
        bf = lambda x: torch.tensor(x).to(torch.bfloat16).to(torch.float64).numpy()
        ref = bf(A) @ bf(B)
        got = Cd.cpu().numpy().T
        assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref)) + 1e-6


def test_backprop_matches_fp64_oracle(eng):
    """Gradients of every layer against the FP64 NumPy MLP (BF16 operand rounding: ~0.5% relative)."""
    import torch
    from sgl_analytic_gb300 import surrogate as S
    mlp = S.MLP(eng, width=64, depth=3, seed=1)
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (512, 8)).astype(np.float32)
    Y = rng.standard_normal((512, 2)).astype(np.float32)
    mlp.stream.synchronize()
    Wh = [w.cpu().numpy() for w in mlp.W]
    bh = [b.cpu().numpy() for b in mlp.b]
    Xd, Yd = S.to_device(eng, X, Y)
    pred = mlp.forward(Xd, keep=True)
    loss, dY = mlp.loss_grad(pred, Yd)
    grads = mlp.backward_step(dY, lr=0.0, wd=0.0)
    mlp.stream.synchronize()
    lref, gref = S.reference_grads(Wh, bh, X, Y)
    assert loss == pytest.approx(lref, rel=1e-2)
    for l, dW, db in grads:
        gw, rw = dW.cpu().numpy(), gref[l][0]
        assert np.linalg.norm(gw - rw) <= 2e-2 * np.linalg.norm(rw)
        assert float(np.sum(gw * rw) / (np.linalg.norm(gw) * np.linalg.norm(rw))) > 0.9995
        assert np.linalg.norm(db.cpu().numpy() - gref[l][1]) <= 2e-2 * np.linalg.norm(gref[l][1])


@pytest.fixture(scope="module")
def small(eng):
    """A small surrogate (3 x 64) trained briefly on 48 planes x 128 q of the FP64 solver."""
    from sgl_analytic_gb300 import planes as P, surrogate as S
    pm = P.PlaneModel()
    th, zl, lnq = S.sample_planes(48, 128, seed=3)
    H = S.solve_planes(eng, pm, th, zl, lnq)
    m1, m2 = S.plane_moments(pm, th, zl)
    sur = S.Surrogate(eng, width=64, depth=3, seed=2)
    hist = sur.train(S.features(th, zl, lnq), S.targets(H, lnq, m1, m2), steps=400, batch=1024, lr=3e-3,
                     log_every=100)
    return pm, sur, hist


def _ensemble(eng, sur, tables):
    import torch
    X = tables.features(eng)
    with torch.cuda.stream(torch.cuda.ExternalStream(eng.stream, device=X.device)):
        Y = torch.stack([m.forward(X) for m in sur.mlps]).contiguous()
    torch.cuda.ExternalStream(eng.stream, device=X.device).synchronize()
    return Y


def test_training_reduces_loss(small):
    _, _, hist = small
    for h in hist:
        assert h[-1] < 0.3 * h[0]


def test_judge_assembly_matches_oracle(eng, small):
    """Judge pass (interpolation, two-moment form, ensemble mean and spread, |Phi| weighting, k band)
    and the FP64 inversion against the NumPy restatement, on uneven instances."""
    from oracle import cfbatch_oracle as CO
    from oracle import sur_oracle as SO
    from sgl_analytic_gb300 import surrogate as S
    from sgl_analytic_gb300._lib import SGL_FP64
    pm, sur, _ = small
    th, zs = S.sample_instances(3, 5)
    tables = S.SweepTables(pm, th, zs, nk=512, nq=32)
    eng.sur_set(tables.inst_plane0, tables.nk, tables.dk, tables.s, tables.dz, tables.mu1, tables.mu2, tables.lnq0,
                tables.hq, tables.nq)
    Y = _ensemble(eng, sur, tables)
    tau = 1e-6
    dis, band = eng.sur_judge(Y, 2, sur.shift, sur.scale, tau)
    lnmu = np.linspace(-1.0, 9.0, 257)
    Pg, L = eng.sur_pdf(lnmu, precision=SGL_FP64, want_lnphi=True)
    Lo, dis_o, band_o = SO.assemble(tables, Y.cpu().numpy(), sur.shift, sur.scale, tau)
    off = 0
    for i, lo in enumerate(Lo):
        lg = L[off:off + lo.size]
        off += lo.size
        assert np.max(np.abs(lg - lo) / (1.0 + np.abs(lo))) < 2e-5
        k = np.arange(lo.size) * tables.dk[i]
        Pref = CO.pdf_from_lnphi(lg, k, lnmu)
        assert np.max(np.abs(Pg[i] - Pref)) <= 1e-10 * np.max(np.abs(Pref))
    assert np.allclose(dis, dis_o, rtol=2e-3, atol=1e-30)
    clear = np.abs(dis_o[:, 1] - tau) > 1e-2 * tau                     # away from the threshold
    assert np.array_equal((band[:, 1] > 0)[clear], (band_o[:, 1] > 0)[clear])
    both = clear & (band[:, 1] > 0) & (band_o[:, 1] > 0)
    assert np.max(np.abs(band[both] - band_o[both]), initial=0) <= 2        # edges may move by a point


def test_judge_fallback_takes_exact_values(eng, small):
    """Planes sent back take the plain FP64 solver's values: all planes (mode "plane", threshold 0)
    reproduce the plain batched solver; "band" takes them on each plane's band of k only."""
    from oracle import sur_oracle as SO
    from sgl_analytic_gb300 import surrogate as S
    from sgl_analytic_gb300._lib import SGL_FP64
    pm, sur, _ = small
    th, zs = S.sample_instances(2, 9, zs=0.5)
    tables = S.SweepTables(pm, th, zs, nk=384, nq=32)
    lnmu = np.linspace(-1.0, 9.0, 129)
    Pall, info = S.judge_sweep(eng, sur, tables, lnmu, threshold=0.0, mode="plane", fallback_precision=SGL_FP64)
    assert info["planes_fraction"] == 1.0 and info["fallback_fraction"] == 1.0
    _, Lall = eng.sur_pdf(lnmu, precision=SGL_FP64, want_lnphi=True)
    Pp, _ = S.plain_pdfs(eng, tables, lnmu, precision=SGL_FP64)
    Lp = eng.cfb_lnphi(SGL_FP64)
    assert np.max(np.abs(Lall - Lp) / (1.0 + np.abs(Lp))) < 1e-12
    assert np.max(np.abs(Pall - Pp)) <= 1e-10 * np.max(np.abs(Pp))
    # band: exact on lo_p <= n < lo_p + nk_p, the surrogate elsewhere
    tau = 1e-7
    Ppre, info = S.judge_sweep(eng, sur, tables, lnmu, threshold=tau, mode="band", fallback_precision=SGL_FP64)
    assert 0 < info["planes_fraction"] and info["fallback_fraction"] < 1
    _, Lpre = eng.sur_pdf(lnmu, precision=SGL_FP64, want_lnphi=True)
    Y = _ensemble(eng, sur, tables)
    off = 0
    for i in range(tables.zs.size):
        nk = int(tables.nk[i])
        k = np.arange(nk) * tables.dk[i]
        ref = np.zeros(nk, complex)
        where = {int(p): j for j, p in enumerate(info["fallback"])}
        for p in range(int(tables.inst_plane0[i]), int(tables.inst_plane0[i + 1])):
            sur_p = np.concatenate([[0], tables.dz[p] * SO.plane_H(tables, Y.cpu().numpy(), p, k[1:], sur.shift,
                                                                     sur.scale).mean(0)])
            if p in where:
                j = where[p]
                lo, nb = int(info["fallback_lo"][j]), int(info["fallback_nk"][j])
                kap, w = tables.plane_cells(p)
                eng.sweep_set_cells(kap, w)
                sur_p[lo:lo + nb] = eng.sweep(k[lo:lo + nb], SGL_FP64)
            ref += sur_p
        assert np.max(np.abs(Lpre[off:off + nk] - ref) / (1.0 + np.abs(ref))) < 2e-5
        off += nk


def test_node_form_matches_plain_solver(eng, small):
    """Planes solved exactly at their log-spaced nodes and interpolated (the judge's node fallback and the
    plain solver's node form) reproduce the plain solver on the full k grid; with threshold 0 the judge
    sends every plane back and equals the node-form plain solver."""
    from sgl_analytic_gb300 import surrogate as S
    from sgl_analytic_gb300._lib import SGL_FP64
    pm, sur, _ = small
    th, zs = S.sample_instances(2, 21, zs=1.0)
    tables = S.SweepTables(pm, th, zs, nk=1024)
    lnmu = np.linspace(-1.0, 9.0, 257)
    Pn, _ = S.plain_node_pdfs(eng, tables, lnmu, precision=SGL_FP64)
    _, Ln = eng.sur_pdf(lnmu, precision=SGL_FP64, want_lnphi=True)
    Pj, info = S.judge_sweep(eng, sur, tables, lnmu, threshold=0.0, mode="nodes", fallback_precision=SGL_FP64)
    _, Lj = eng.sur_pdf(lnmu, precision=SGL_FP64, want_lnphi=True)
    assert info["planes_fraction"] == 1.0
    # the same node values (held as normalised float32 residuals: one rounding of the scaling apart) where
    # |Phi| does not underflow float32 (beyond, no weighted spread exceeds 0 and the band stops)
    live = Ln.real > -80.0
    assert np.max(np.abs(Lj - Ln)[live] / (1.0 + np.abs(Ln[live]))) < 1e-6
    l1j, _ = S.pdf_errors(Pj, Pn, lnmu)
    assert l1j.max() < 1e-7
    Pp, _ = S.plain_pdfs(eng, tables, lnmu, precision=SGL_FP64)
    Lp = eng.cfb_lnphi(SGL_FP64)
    # node interpolation: float32 node residuals, 4-point Lagrange in ln q
    assert np.max(np.abs(Ln - Lp) / (1.0 + np.abs(Lp))) < 1e-5
    l1, _ = S.pdf_errors(Pn, Pp, lnmu)
    assert l1.max() < 1e-5


def test_fused_inference_matches_layerwise_forward(eng):
    """sgl_mlp_infer (one fused kernel, activations on chip) against the layer-by-layer forward of the
    same network (the training forward's arithmetic), on a ragged number of rows."""
    import torch
    from sgl_analytic_gb300 import surrogate as S
    mlp = S.MLP(eng, width=256, depth=6, seed=5)
    rng = np.random.default_rng(4)
    for n in (1, 300, 4097):
        (Xd,) = S.to_device(eng, rng.uniform(-1, 1, (n, 8)).astype(np.float32))
        ref = mlp.forward(Xd)
        got = mlp.infer(Xd)
        mlp.stream.synchronize()
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        assert g.shape == (n, 2)
        assert np.max(np.abs(g - r)) <= 1e-4 * max(1.0, np.max(np.abs(r))), n
