"""The FP64 oracle (oracle/) pinned against the reference's own outputs.

Golden vectors: tests/golden/ref_zs1_sub.npz, produced by the reference's NumPy code on the
committed population (tests/golden/make_golden.py), and the reference's stored golden PDF
tests/golden/pdf_zs1.json (its tests/reference/, checked by its tests/test_reference.py at
max|dP|/peak <= 1e-9).
"""
import json

import numpy as np
import pytest

from oracle import invert_oracle as IO
from oracle import lam_oracle as LO
from oracle import vp_oracle as VO
from tests.conftest import FULL_FIXTURE, GOLDEN, VP_FULL

TOL_LN = 1e-10          # max |d ln Phi| (spec FP64 bar)
TOL_PEAK = 1e-9         # max |dP| / peak (the reference's own regression tolerance)


def oracle_for(pop, xi, method="sep"):
    X = LO.XiGroups(pop.groups(), pop.ce_k, pop.ce_g) if xi else None
    return LO.OracleLam(pop.w0, pop.k0, pop.g0, pop.ig, pop.fe_g, pop.V, X, method=method)


def test_psi1_direct_matches_reference(pop_sub, ref_sub):
    lam = oracle_for(pop_sub, False, "direct")
    L = lam(ref_sub["kk"], ref_sub["kg"])
    assert np.max(np.abs(L - ref_sub["psi1_grid"])) <= TOL_LN


def test_psi1_separable_matches_reference_direct(pop_sub, ref_sub):
    # the separable path depends on the full k_gamma extent (node placement): evaluate the
    # sub-sampled k_kappa rows against the FULL k_gamma axis, compare every 32nd column
    kg_full = np.linspace(0.0, 808.3706243177588, 2687)
    lam = oracle_for(pop_sub, False, "sep")
    L = lam.psi1_sep(ref_sub["kk"], kg_full)[:, ::32]
    assert np.max(np.abs(L - ref_sub["psi1_grid"])) <= TOL_LN


def test_probe_lines_and_sigma(pop_sub, ref_sub):
    lam = oracle_for(pop_sub, False, "direct")
    ks = ref_sub["probe_k"]
    assert np.max(np.abs(lam(ks, np.zeros(1))[:, 0] - ref_sub["psi1_line_k"])) <= TOL_LN
    assert np.max(np.abs(lam(np.zeros(1), ks)[0, :] - ref_sub["psi1_line_g"])) <= TOL_LN
    assert lam.sigma() == pytest.approx(float(ref_sub["sigma1"]), rel=1e-14)
    assert oracle_for(pop_sub, True).sigma() == pytest.approx(float(ref_sub["sigmax"]), rel=1e-14)


def test_xi_term_matches_reference(pop_sub, ref_sub):
    lam = oracle_for(pop_sub, True)
    Q = lam.qxi(ref_sub["kkc"], ref_sub["kgc"])
    Qr = ref_sub["xi_coarse"]
    assert np.max(np.abs(Q - Qr)) <= TOL_LN * max(1.0, np.max(np.abs(Qr)))
    ks = ref_sub["probe_k"]
    assert np.max(np.abs(lam.qxi(ks, np.zeros(1))[:, 0] - ref_sub["xi_line_k"])) <= TOL_LN
    assert np.max(np.abs(lam.qxi(np.zeros(1), ks)[0, :] - ref_sub["xi_line_g"])) <= TOL_LN
    # full composition on a small grid (exact xi term)
    L = lam(ref_sub["kk"][:20], ref_sub["kg"][:20])
    assert np.max(np.abs(L - ref_sub["lamx_grid"])) <= TOL_LN


def _check_pdf(P, Pref, x):
    peak = np.max(Pref)
    assert np.max(np.abs(P - Pref)) / peak <= TOL_PEAK
    assert np.trapezoid(np.abs(P - Pref), x) <= 1e-9


def test_invert_chain_matches_reference(pop_sub, ref_sub):
    """Psi_1 + xi subset through the whole inversion (separable Lambda, as the reference's default)."""
    lam = oracle_for(pop_sub, True, "sep")
    x = ref_sub["xi_out"]
    _, P, meta = IO.invert(lam, lam.sigma(), x)
    g = meta["grid"]
    ref_grid = ref_sub["pdfx_grid"]
    assert [g["nk_k"], g["nk_g"], g["n_kap"], g["n_gam"]] == [int(ref_grid[i]) for i in (0, 1, 4, 5)]
    _check_pdf(P, ref_sub["pdfx_P"], x)
    np.testing.assert_allclose([meta["mean"], meta["var"], meta["skew"], meta["sigmaDL"]],
                               ref_sub["pdfx_moments"], rtol=1e-8)


@pytest.mark.skipif(not FULL_FIXTURE.exists(), reason="full z_s=1 population (290 MB) not present")
def test_full_chain_matches_stored_golden_pdf():
    """All 201 xi groups: the oracle reproduces the reference's stored z_s=1 PDF."""
    lam = LO.oracle_from_npz(FULL_FIXTURE)
    ref = json.load(open(GOLDEN / "pdf_zs1.json"))
    x = np.concatenate([ref["xi"], ref["xi_tail"]])
    _, P, meta = IO.invert(lam, lam.sigma(), x)
    P0 = np.concatenate([ref["P_s"], ref["P_s_tail"]])
    assert np.max(np.abs(P - P0)) / P0.max() <= TOL_PEAK
    assert meta["grid"]["nk_k"] == ref["grid"]["nk_k"] and meta["grid"]["nk_g"] == ref["grid"]["nk_g"]


def test_vp_oracle_matches_reference_sub_golden():
    """vp closure, shells 0-5: the oracle's ln R against the reference's _fused_groups +
    _chain_recursion on the same sub-closure (5 x 4 points)."""
    d = dict(np.load(GOLDEN / "vp_zs1_sub.npz"))
    L = VO.lnR(d, d["kv"], d["qv"])
    assert np.all(np.abs(L - d["lnR"]) <= 1e-15 + 1e-12 * np.abs(d["lnR"]))


def test_vp_oracle_unwraps_like_numpy():
    """q_xi's phase is unwrapped along k_kappa at the first k_gamma column, then along k_gamma."""
    d = dict(np.load(GOLDEN / "vp_zs1_sub.npz"))
    kv, qv = np.array([0.0, 300.0, 900.0]), np.array([0.0, 100.0])
    Q = VO.qxi(d, kv, qv)
    L = VO.lnR(d, kv, qv)
    assert np.allclose(np.exp(1j * Q.imag), np.exp(1j * L.imag), atol=1e-12)
    assert np.allclose(Q.real, L.real - 0.25 * float(d["shear_var"]) * qv[None, :] ** 2, rtol=0, atol=1e-15)


@pytest.mark.skipif(not VP_FULL.exists(), reason="full z_s=1 vp closure (34 MB) not present")
def test_vp_oracle_matches_reference_full_closure_probe():
    """All 67 shells: the oracle against FusedVP.lnR_blocked and Closure.lnR_ref on 3 x 3 points."""
    d = dict(np.load(VP_FULL))
    p = np.load(GOLDEN / "vp_zs1_full_lnR_probe.npz")
    L = VO.lnR(d, p["kv"], p["qv"])
    for key in ("fused", "ref"):
        assert np.all(np.abs(L - p[key]) <= 1e-13 + 1e-10 * np.abs(p[key])), key


def test_vp_oracle_mirrored_closure_gives_same_lnR():
    """Right-clipped rates: relabelling the states j -> 47 - j leaves ln R unchanged."""
    from tests.test_gpu_vp import mirrored
    d = dict(np.load(GOLDEN / "vp_zs1_sub.npz"))
    kv, qv = np.array([0.0, 40.0, 900.0]), np.array([0.0, 150.0, 600.0])
    L = VO.lnR(d, kv, qv)
    Lm = VO.lnR(mirrored(d), kv, qv)
    assert np.all(np.abs(L - Lm) <= 1e-14 + 1e-11 * np.abs(L))


def test_mlp_gradient_oracle_matches_finite_differences():
    """The FP64 NumPy back-propagation used to check the GPU gradients, against central differences."""
    from sgl_analytic_gb300.surrogate import reference_grads
    rng = np.random.default_rng(1)
    sizes = [8, 16, 16, 2]
    W = [rng.standard_normal((a, c)) * 0.5 for a, c in zip(sizes[:-1], sizes[1:])]
    b = [rng.standard_normal(c) * 0.1 for c in sizes[1:]]
    X, Y = rng.uniform(-1, 1, (32, 8)), rng.standard_normal((32, 2))
    _, g = reference_grads(W, b, X, Y)
    h = 1e-6
    for l in range(3):
        for (i, j) in [(0, 0), (1, 1), (2, 1)]:
            Wp = [w.copy() for w in W]; Wp[l][i, j] += h
            Wm = [w.copy() for w in W]; Wm[l][i, j] -= h
            fd = (reference_grads(Wp, b, X, Y)[0] - reference_grads(Wm, b, X, Y)[0]) / (2 * h)
            assert abs(fd - g[l][0][i, j]) <= 1e-6 * max(1.0, abs(fd))


def test_surrogate_targets_round_trip():
    """The surrogate's residual targets over the two-moment form invert exactly, the plane moments in
    closed form equal the cells' sums, and arg(-H) never wraps."""
    from sgl_analytic_gb300 import planes as P, surrogate as S
    m = P.PlaneModel()
    bg = P.Background(P.FIDUCIAL)
    S_, w = m.cells(bg, 0, 0.5)
    mu1, mu2 = m.moments(bg, 0, np.array([0.5]))
    assert mu1[0] == pytest.approx(np.sum(w * S_), rel=1e-12)
    assert mu2[0] == pytest.approx(np.sum(w * S_ * S_), rel=1e-12)
    q = np.geomspace(1e-4, 4e3, 40)
    H = np.array([np.sum(w * (np.expm1(1j * qq * S_) - 1j * qq * S_)) for qq in q])[None, :]
    R = S.targets(H, np.log(q)[None, :], mu1, mu2)
    assert np.all(np.abs(np.diff(np.angle(-H[0]))) < 1.0)              # no 2 pi wrap of the phase
    assert np.max(np.abs(R)) < 10.0                                     # an O(1) residual
    assert np.max(np.abs(S.untarget(R, np.log(q)[None, :], mu1, mu2) - H.ravel()) / np.abs(H.ravel())) < 1e-9
