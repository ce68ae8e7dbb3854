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


def test_training_reduces_loss_and_judge_falls_back_exactly(eng):
    from sgl_analytic_gb300 import surrogate as S
    model = S.PlaneModel()
    th, zl, lnk = S.sample_inputs(24, 256, seed=3)
    L = S.solve_planes(eng, model, th, zl, lnk)
    sur = S.Surrogate(eng, width=64, depth=3, seed=2)
    hist = sur.train(S.features(th, zl, lnk), S.targets(L), epochs=8, batch=1024, lr=3e-3)
    for h in hist:
        assert h[-1] < 0.5 * h[0]
    lam, bad = S.judge(eng, model, sur, th, zl, lnk, threshold=1e-5)
    assert bad.any()
    assert np.array_equal(lam[bad], L[bad])                  # fallback planes are the solver's values
