"""The allocation-free entry point sgl_cf_kappa_noalloc, called through the C ABI.

It is meant for callers that may not allocate device memory themselves (their device budget is
handed to their own pool or caching allocator, or their runtime forbids third-party
allocations); it keeps its partial sums in a fixed 8 MiB device array instead.  Here the inputs
and outputs are device buffers that the test owns (allocated by torch), and the result is
checked against the regular entry point sgl_lnphi at k_gamma = 0 on two calls in a row, with
different grids, so that the second call cannot pass on what the first one left in the shared
array.  This file is collected last, so a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10          # the FP64 bar of the parity tests (relative 1e-12 where |ln Phi| > 100)


def _close(a, b):
    return bool(np.all(np.abs(a - b) <= np.maximum(TOL, 1e-12 * np.abs(b))))


def _call(L, kk_h, k0, w0, n_cells, dev, torch):
    import ctypes as C
    from sgl_analytic_gb300._lib import SGL_OK
    kk = torch.tensor(kk_h, dtype=torch.float64, device=dev)
    out_re = torch.full((kk_h.size,), np.nan, dtype=torch.float64, device=dev)
    out_im = torch.full((kk_h.size,), np.nan, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = L.sgl_cf_kappa_noalloc(C.c_void_p(kk.data_ptr()), kk_h.size, C.c_void_p(k0.data_ptr()),
                                C.c_void_p(w0.data_ptr()), n_cells, C.c_void_p(out_re.data_ptr()),
                                C.c_void_p(out_im.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == SGL_OK
    torch.cuda.synchronize(dev)
    return out_re.cpu().numpy() + 1j * out_im.cpu().numpy()


def test_noalloc_matches_regular_entry_point_on_two_calls(pop_sub):
    torch = pytest.importorskip("torch")
    from sgl_analytic_gb300 import Lam
    from sgl_analytic_gb300._lib import lib

    assert pop_sub.V == 0.0                      # sgl_lnphi at k_gamma = 0 is then exactly this sum
    lam = Lam(pop_sub, xi=False)                 # regular entry point (context, arena scratch)
    L = lib()
    dev = torch.device("cuda", 0)
    k0 = torch.tensor(pop_sub.k0, dtype=torch.float64, device=dev)
    w0 = torch.tensor(pop_sub.w0, dtype=torch.float64, device=dev)
    grids = [np.linspace(0.0, 1010.4632803971984, 1683),          # the z_s=1 k_kappa axis
             np.geomspace(1e-3, 2.0e3, 777)[::-1].copy()]           # another size and order
    for kk_h in grids:
        got = _call(L, kk_h, k0, w0, pop_sub.n_cells, dev, torch)
        ref = lam(kk_h, np.zeros(1))[:, 0]
        assert np.all(np.isfinite(got))
        assert _close(got, ref), float(np.max(np.abs(got - ref)))


def test_noalloc_at_the_size_limit(pop_sub):
    """The largest grid the fixed scratch takes (32768 k-points: every chunk's partials fill the
    array to its end), on a 3000-cell slice of the population, against the regular entry point."""
    torch = pytest.importorskip("torch")
    from dataclasses import replace

    from sgl_analytic_gb300 import Lam
    from sgl_analytic_gb300._lib import lib
    sl = slice(0, 3000)
    pop = replace(pop_sub, w0=pop_sub.w0[sl].copy(), k0=pop_sub.k0[sl].copy(), g0=pop_sub.g0[sl].copy(),
                  ig=pop_sub.ig[sl].copy())
    lam = Lam(pop, xi=False)
    dev = torch.device("cuda", 0)
    k0 = torch.tensor(pop.k0, dtype=torch.float64, device=dev)
    w0 = torch.tensor(pop.w0, dtype=torch.float64, device=dev)
    kk_h = np.linspace(0.0, 1500.0, 32768)
    got = _call(lib(), kk_h, k0, w0, pop.n_cells, dev, torch)
    ref = lam(kk_h, np.zeros(1))[:, 0]
    assert np.all(np.isfinite(got))
    assert _close(got, ref), float(np.max(np.abs(got - ref)))


def test_noalloc_rejects_oversized_grid():
    from sgl_analytic_gb300._lib import SGL_ERR_VALUE, lib
    L = lib()
    st = L.sgl_cf_kappa_noalloc(ctypes.c_void_p(1), 32769, ctypes.c_void_p(1), ctypes.c_void_p(1), 1,
                                ctypes.c_void_p(1), ctypes.c_void_p(1), None)
    assert st == SGL_ERR_VALUE
    buf = ctypes.create_string_buffer(256)
    L.sgl_last_error(None, buf, 256)
    assert b"32768" in buf.value
