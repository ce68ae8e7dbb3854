"""GPU checks of the batched CF solver (sgl_cfb_*): one persistent launch over uneven instances
(plane counts, k grids, gauss and vp closures), the tile autotuner and the CUDA-graph replay,
against the FP64 NumPy oracle (oracle/cfbatch_oracle.py).

Tolerances: FP64 ln Phi within 1e-10 (1 + |ln Phi|) where |Phi| > 1e-30 and the FP64 PDF within 1e-9
of its peak; mixed ln Phi within 1e-6 (1 + |ln Phi|) there, mixed PDF L1 <= 1e-4 and within 1e-5 of peak.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    from sgl_analytic_gb300.cfbatch import make_batch
    return make_batch(7, seed=5, nm=6, nb=6, nk_range=(300, 1300), nk_step=1, max_planes=9)


@pytest.fixture(scope="module")
def eng(small):
    from sgl_analytic_gb300._lib import Engine
    e = Engine(0)
    e.cfb_set(small.arrays())
    return e


def _split(small, L):
    offs = np.concatenate([[0], np.cumsum(small.nk.astype(np.int64))])
    return [L[offs[i]:offs[i + 1]] for i in range(small.n_inst)]


def _close(a, b, rtol):
    """|e^a - e^b| relative to |e^b| and the real parts, where |Phi| > 1e-30 (the imaginary part of
    the vp closure's logarithm is a principal branch)."""
    keep = b.real > np.log(1e-30)
    da = np.abs(np.exp(a[keep] - b[keep]) - 1.0)
    return float(np.max(da)) if keep.any() else 0.0


def test_uneven_batch_lnphi_fp64_matches_oracle(small, eng):
    from oracle import cfbatch_oracle as O
    from sgl_analytic_gb300._lib import SGL_FP64
    assert len(set(small.nk.tolist())) > 3 and set(small.closure.tolist()) == {0, 1}
    L = _split(small, eng.cfb_lnphi(SGL_FP64))
    for i in range(small.n_inst):
        ref = O.lnphi(small, i)
        assert _close(L[i], ref, 1e-10) <= 1e-10 * (1 + np.max(np.abs(ref.real))), i


def test_mixed_lnphi_and_pdfs(small, eng):
    from oracle import cfbatch_oracle as O
    from sgl_analytic_gb300._lib import SGL_FP64, SGL_MIXED
    Lm = _split(small, eng.cfb_lnphi(SGL_MIXED))
    for i in range(small.n_inst):
        ref = O.lnphi(small, i)
        assert _close(Lm[i], ref, 1e-6) <= 1e-6 * (1 + np.max(np.abs(ref.real))), i
    lnmu = np.linspace(-0.4, 1.5, 777)
    P64, _ = eng.cfb_pdf(lnmu, SGL_FP64, use_graph=False)
    Pm, _ = eng.cfb_pdf(lnmu, SGL_MIXED, use_graph=False)
    for i in range(small.n_inst):
        ref = O.pdf_lnmu(small, i, lnmu)
        peak = np.max(np.abs(ref))
        assert np.max(np.abs(P64[i] - ref)) <= 1e-9 * peak, i
        assert np.max(np.abs(Pm[i] - ref)) <= 1e-5 * peak, i
        assert np.trapezoid(np.abs(Pm[i] - ref), lnmu) <= 1e-4


def test_graph_replay_and_tuning(small, eng):
    from sgl_analytic_gb300._lib import SGL_MIXED
    kt, cps = eng.cfb_tune(SGL_MIXED)
    assert kt in (64, 128, 256) and cps >= 1
    lnmu = np.linspace(-0.4, 1.5, 300)
    direct, _ = eng.cfb_pdf(lnmu, SGL_MIXED, use_graph=False)
    g1, _ = eng.cfb_pdf(lnmu, SGL_MIXED, use_graph=True)      # captured
    g2, _ = eng.cfb_pdf(lnmu, SGL_MIXED, use_graph=True)      # replayed
    np.testing.assert_array_equal(g1, direct)
    np.testing.assert_array_equal(g2, direct)


def test_bad_batches_raise():
    from sgl_analytic_gb300._lib import Engine
    from sgl_analytic_gb300.cfbatch import make_batch
    b = make_batch(2, seed=1, nm=4, nb=4, nk_range=(64, 128), nk_step=1, max_planes=3).arrays()
    e = Engine(0)
    bad = dict(b, nk=np.array([1, 64], np.int32))
    with pytest.raises(ValueError):
        e.cfb_set(bad)
    bad = dict(b, inst_plane0=np.array([0, 3, 3], np.int32))
    with pytest.raises(ValueError):
        e.cfb_set(bad)
    with pytest.raises(RuntimeError):
        e.cfb_lnphi()                    # nothing set on this engine
