"""GPU parity of the one-dimensional compensated CF sweep (the synthetic plane x mass x impact-parameter
microbenchmark and the kappa part of Psi_1)."""
import numpy as np
import pytest

from oracle import lam_oracle as LO

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from sgl_analytic_gb300._lib import Engine
    return Engine(0)


def test_sweep_equals_lnphi_on_kappa_axis(eng, pop_sub):
    """On the reference's z_s=1 cells (V = 0, no xi term): the sweep is ln Phi(k, 0)."""
    from sgl_analytic_gb300 import Lam
    lam = Lam(pop_sub, xi=False)
    kk = np.linspace(0.0, 1010.4632803971984, 1683)[::7]
    eng.sweep_set_cells(pop_sub.k0, pop_sub.w0)
    got = eng.sweep(kk)
    ref = lam(kk, np.zeros(1))[:, 0]
    assert np.all(np.abs(got - ref) <= np.maximum(1e-10, 1e-12 * np.abs(ref)))


def test_synthetic_sweep_fp64_and_mixed_vs_oracle(eng):
    from sgl_analytic_gb300._lib import SGL_MIXED
    from sgl_analytic_gb300.workloads import cf_sweep_problem
    kap, w, kk = cf_sweep_problem()
    kap, w = kap[::61], w[::61]                     # 275k cells of the 16.8M
    kk = kk[::331]                                  # 50 k in [1e-2, 1e6]
    eng.sweep_set_cells(kap, w)
    ref, mag = LO.cf_sweep(kk, kap, w)
    got = eng.sweep(kk)
    assert np.all(np.abs(got - ref) <= 1e-10 + 1e-13 * mag)
    mix = eng.sweep(kk, SGL_MIXED)
    assert np.all(np.abs(mix - ref) <= 1e-6 * mag)


def test_measured_peaks_are_positive(eng):
    f64, f32 = eng.measure_peak(True), eng.measure_peak(False)
    assert 0.1 < f64 < 1e3 and 1.0 < f32 < 1e4
