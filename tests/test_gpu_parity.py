"""GPU parity: the CUDA path (through the C ABI) against the reference's own outputs and the oracle.

Tolerances (the benchmark spec): FP64 path max|d ln Phi| <= 1e-10 and max|dP|/peak <= 1e-9 (the
reference's regression tolerance); mixed path PDF L1 <= 1e-4 and tail relative error <= 1e-3.
"""
import json

import numpy as np
import pytest

from tests.conftest import FULL_FIXTURE, GOLDEN

pytestmark = pytest.mark.gpu

TOL_LN = 1e-10
TOL_PEAK = 1e-9
KG_FULL = np.linspace(0.0, 808.3706243177588, 2687)
KK16 = np.linspace(0.0, 1010.4632803971984, 1683)[::16]     # 106 rows: 106 x 2687 > 200000 points


@pytest.fixture(scope="module")
def lam1(pop_sub):
    from sgl_analytic_gb300 import Lam
    return Lam(pop_sub, xi=False)


@pytest.fixture(scope="module")
def lamx(pop_sub):
    from sgl_analytic_gb300 import Lam
    return Lam(pop_sub, xi=True)


def test_sigma(lam1, lamx, ref_sub):
    assert lam1.sigma() == pytest.approx(float(ref_sub["sigma1"]), rel=1e-13)
    assert lamx.sigma() == pytest.approx(float(ref_sub["sigmax"]), rel=1e-13)


def test_psi1_direct_small_grid(lam1, ref_sub):
    L = lam1(ref_sub["kk"], ref_sub["kg"])            # 4452 points: direct sums
    assert np.max(np.abs(L - ref_sub["psi1_grid"])) <= TOL_LN


def _ln_close(a, b):
    """max|d ln Phi| <= 1e-10 where |ln Phi| <= 100; beyond (|Phi| < e^-100, far past the k-reach)
    the bar is 1e-12 relative: the FP64 roundoff of sums whose weights total 3.7e6 (ulp 4.7e-10)."""
    tol = np.maximum(TOL_LN, 1e-12 * np.abs(b))
    return bool(np.all(np.abs(a - b) <= tol))


def test_psi1_probe_lines(lam1, ref_sub):
    ks = ref_sub["probe_k"]
    assert _ln_close(lam1(ks, np.zeros(1))[:, 0], ref_sub["psi1_line_k"])
    assert _ln_close(lam1(np.zeros(1), ks)[0, :], ref_sub["psi1_line_g"])


def test_psi1_separable_full_width(lam1, ref_sub):
    # >= 200000 points: the separable sweep + Chebyshev GEMMs + direct-tail GEMM
    L = lam1(KK16, KG_FULL)
    assert L.shape == (KK16.size, KG_FULL.size)
    assert np.max(np.abs(L[::2, ::32] - ref_sub["psi1_grid"])) <= TOL_LN


def test_cells_below_their_gamma_bin(pop_sub):
    """Cells whose gamma lies below their bin's lower edge (the reference's z_s = 10 population
    has two: gamma = 0 in a bin starting at 2.9e-3, and 7e-10 in [1e-9, 1.08e-9)).  The separable
    plan keeps the reference's negative sub-bin index (truncation toward zero, no lower clamp) and
    orders the sub-bins by their lower edges; the GPU matches the oracle's separable form."""
    import dataclasses

    from oracle import lam_oracle as LO
    from sgl_analytic_gb300 import Lam
    g0 = pop_sub.g0.copy()
    lo = pop_sub.fe_g[pop_sub.ig]
    c0 = int(np.argmax(lo))                    # highest bin: gamma = 0 lies many sub-bins below
    c1 = int(np.argmax(np.where(pop_sub.ig == np.median(pop_sub.ig).astype(int), lo, -1.0)))
    g0[c0] = 0.0
    g0[c1] = 0.7 * lo[c1]
    assert np.sum(g0 < lo) == 2
    pop = dataclasses.replace(pop_sub, g0=g0)
    L = Lam(pop, xi=False)(KK16, KG_FULL)
    O = LO.OracleLam(pop.w0, pop.k0, g0, pop.ig, pop.fe_g, pop.V, None, method="sep")
    Lo = O(KK16, KG_FULL)
    assert _ln_close(L[::3, ::17], Lo[::3, ::17])


def test_psi1_separable_mixed_precision(lam1, ref_sub):
    from sgl_analytic_gb300._lib import SGL_MIXED
    Lm = lam1.engine.lnphi(KK16, KG_FULL, SGL_MIXED)[::2, ::32]
    Lr = ref_sub["psi1_grid"]
    # Phi = exp(ln Phi) agrees to 1e-5 absolute; ln Phi to 1e-3 where |Phi| > 1e-6
    assert np.max(np.abs(np.exp(Lm) - np.exp(Lr))) <= 1e-5
    big = np.abs(np.exp(Lr)) > 1e-6
    assert np.max(np.abs(Lm - Lr)[big]) <= 1e-3


def test_xi_term_exact(lamx, ref_sub):
    Q = lamx.engine.xi_term(ref_sub["kkc"], ref_sub["kgc"])
    Qr = ref_sub["xi_coarse"]
    assert np.max(np.abs(Q - Qr)) <= TOL_LN * max(1.0, np.max(np.abs(Qr)))
    ks = ref_sub["probe_k"]
    assert np.max(np.abs(lamx.engine.xi_term(ks, np.zeros(1))[:, 0] - ref_sub["xi_line_k"])) <= TOL_LN
    assert np.max(np.abs(lamx.engine.xi_term(np.zeros(1), ks)[0, :] - ref_sub["xi_line_g"])) <= TOL_LN


def test_xi_term_mixed_vs_fp64(lamx, ref_sub):
    """The mixed path's compensated m=0 form (sum (cos-1) T + U (J0-1)) in FP32 vs the FP64 term."""
    from sgl_analytic_gb300._lib import SGL_MIXED
    Q = lamx.engine.xi_term(ref_sub["kkc"], ref_sub["kgc"], SGL_MIXED)
    Qr = ref_sub["xi_coarse"]
    assert np.max(np.abs(Q - Qr)) <= 1e-5 * max(1.0, np.max(np.abs(Qr)))


def _groups_with_rows(pop_sub, rows):
    """pop_sub with every xi group given `rows` rows: the first rows of each group, and beyond its
    own rows, copies of them scaled by 0.9^(pass) (each group's rows are nrow x (nidx + 1),
    row-major; the last column is the residual)."""
    from dataclasses import replace
    nr, nc = pop_sub.xg_nrow.astype(np.int64), pop_sub.xg_nidx.astype(np.int64) + 1
    off = np.concatenate([[0], np.cumsum(nr * nc)])
    blocks = []
    for g in range(nr.size):
        R = pop_sub.xg_rows[off[g]:off[g + 1]].reshape(nr[g], nc[g])
        blocks.append(np.concatenate([R[r % nr[g]] * 0.9 ** (r // nr[g]) for r in range(rows)]))
    return replace(pop_sub, xg_nrow=np.full(nr.size, rows, np.int32), xg_rows=np.concatenate(blocks))


@pytest.mark.parametrize("rows", [5, 17, 37, 48, 60])
def test_xi_term_mixed_few_rows(pop_sub, ref_sub, rows):
    """Groups of 5 and 17 rows (fewer than one warp of row tasks), 37 (the reference's longest
    groups at z_s = 1), 48 (the fused kernel's longest: fewer entries per chunk) and 60 (split into
    two groups of 30 rows by the engine): the mixed xi term (fused tcgen05 kernel) against the FP64
    term on the coarse grid, and for the longer groups the FP64 term against the oracle."""
    from oracle import lam_oracle as LO
    from sgl_analytic_gb300 import Lam
    from sgl_analytic_gb300._lib import SGL_FP64, SGL_MIXED
    pop = _groups_with_rows(pop_sub, rows)
    lam = Lam(pop, xi=True, xi_prune=0.0)          # no pruning: the oracle below sees every row
    Q64 = lam.engine.xi_term(ref_sub["kkc"], ref_sub["kgc"], SGL_FP64)
    Qmx = lam.engine.xi_term(ref_sub["kkc"], ref_sub["kgc"], SGL_MIXED)
    assert np.max(np.abs(Qmx - Q64)) <= 1e-5 * max(1.0, np.max(np.abs(Q64)))
    if rows > 36:
        X = LO.XiGroups(pop.groups(), pop.ce_k, pop.ce_g, prune=0.0)
        ol = LO.OracleLam(pop.w0, pop.k0, pop.g0, pop.ig, pop.fe_g, pop.V, X)
        Qo = ol.qxi(ref_sub["kkc"][::10], ref_sub["kgc"][::10])
        assert np.max(np.abs(Q64[::10, ::10] - Qo)) <= TOL_LN * max(1.0, np.max(np.abs(Qo)))


def test_lambda_full_grid_mixed_vs_fp64(lamx):
    from sgl_analytic_gb300._lib import SGL_FP64, SGL_MIXED
    L64 = lamx.engine.lnphi(KK16, KG_FULL, SGL_FP64)
    Lmx = lamx.engine.lnphi(KK16, KG_FULL, SGL_MIXED)
    assert np.max(np.abs(np.exp(Lmx) - np.exp(L64))) <= 1e-5


def test_pdf_mixed_psi1_only(lam1, ref_sub):
    from sgl_analytic_gb300 import invert
    x = ref_sub["xi_out"]
    _, P, _ = invert(lam1, lam1.sigma(), xi_out=x, tail_box=True, phi_tol=1e-8, precision="mixed")
    dpeak, l1, rel_tail = _pdf_errors(P, ref_sub["pdf1_P"], x)
    assert l1 <= 1e-4 and rel_tail <= 1e-3, (dpeak, l1, rel_tail)


def test_lambda_with_xi_small_grid(lamx, ref_sub):
    L = lamx(ref_sub["kk"][:20], ref_sub["kg"][:20])
    assert np.max(np.abs(L - ref_sub["lamx_grid"])) <= TOL_LN


def test_lambda_with_xi_interpolated_matches_oracle(lamx, pop_sub, ref_sub):
    """Full-width grid: separable Psi_1 + 101^2 coarse xi term + not-a-knot bicubic spline."""
    from oracle import lam_oracle as LO
    X = LO.XiGroups(pop_sub.groups(), pop_sub.ce_k, pop_sub.ce_g)
    orc = LO.OracleLam(pop_sub.w0, pop_sub.k0, pop_sub.g0, pop_sub.ig, pop_sub.fe_g, pop_sub.V, X)
    kk = KK16
    L = lamx(kk, KG_FULL)
    Lo = orc(kk, KG_FULL)
    assert np.max(np.abs(L - Lo)) <= TOL_LN


def _pdf_errors(P, Pref, x):
    peak = np.max(Pref)
    l1 = np.trapezoid(np.abs(P - Pref), x)
    tail = x > 1.0
    sig = np.abs(Pref[tail]) > 1e-6 * peak
    rel_tail = np.max(np.abs(P[tail][sig] - Pref[tail][sig]) / np.abs(Pref[tail][sig])) if sig.any() else 0.0
    return np.max(np.abs(P - Pref)) / peak, l1, rel_tail


@pytest.mark.parametrize("which", ["pdf1", "pdfx"])
def test_pdf_fp64_matches_reference(which, lam1, lamx, ref_sub):
    from sgl_analytic_gb300 import invert
    lam = lam1 if which == "pdf1" else lamx
    x = ref_sub["xi_out"]
    _, P, meta = invert(lam, lam.sigma(), xi_out=x, tail_box=True, phi_tol=1e-8, n_xi_wide=500)
    g = meta["grid"]
    rg = ref_sub[which + "_grid"]
    assert [g["nk_k"], g["nk_g"], g["n_kap"], g["n_gam"]] == [int(rg[i]) for i in (0, 1, 4, 5)]
    assert g["k_k_max"] == pytest.approx(rg[2], rel=1e-14) and g["k_g_max"] == pytest.approx(rg[3], rel=1e-14)
    dpeak, l1, _ = _pdf_errors(P, ref_sub[which + "_P"], x)
    assert dpeak <= TOL_PEAK and l1 <= 1e-9
    np.testing.assert_allclose([meta["mean"], meta["var"], meta["skew"], meta["sigmaDL"]],
                               ref_sub[which + "_moments"], rtol=1e-8)


def test_pdf_mixed_matches_reference(lamx, ref_sub):
    from sgl_analytic_gb300 import invert
    x = ref_sub["xi_out"]
    _, P, _ = invert(lamx, lamx.sigma(), xi_out=x, tail_box=True, phi_tol=1e-8, precision="mixed")
    dpeak, l1, rel_tail = _pdf_errors(P, ref_sub["pdfx_P"], x)
    assert l1 <= 1e-4 and rel_tail <= 1e-3, (dpeak, l1, rel_tail)


def test_pdf_is_deterministic(lamx, ref_sub):
    from sgl_analytic_gb300 import invert
    x = ref_sub["xi_out"][::50]
    a = invert(lamx, lamx.sigma(), xi_out=x, phi_tol=1e-8)[1]
    b = invert(lamx, lamx.sigma(), xi_out=x, phi_tol=1e-8)[1]
    assert np.array_equal(a, b)


def test_bad_input_raises_value_error(lam1):
    with pytest.raises(ValueError):
        lam1(np.array([np.nan, 1.0]), np.array([0.0, 1.0]))
    with pytest.raises(ValueError):
        lam1(np.array([1.0]), np.array([-1.0]))


@pytest.mark.skipif(not FULL_FIXTURE.exists(), reason="full z_s=1 population (290 MB) not shipped")
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_full_chain_matches_stored_golden_pdf(precision):
    """All 201 xi groups: GPU vs the reference's stored z_s=1 golden PDF."""
    from sgl_analytic_gb300 import Lam, Population, invert
    lam = Lam(Population.load(FULL_FIXTURE), xi=True)
    ref = json.load(open(GOLDEN / "pdf_zs1.json"))
    x = np.concatenate([ref["xi"], ref["xi_tail"]])
    _, P, meta = invert(lam, lam.sigma(), xi_out=x, phi_tol=1e-8, precision=precision)
    P0 = np.concatenate([ref["P_s"], ref["P_s_tail"]])
    dpeak, l1, rel_tail = _pdf_errors(P, P0, x)
    if precision == "fp64":
        assert dpeak <= TOL_PEAK
    else:
        assert l1 <= 1e-4 and rel_tail <= 1e-3


def test_api_generate_pdf_lnmu_matches_reference(ref_sub):
    """The drop-in API end to end (population given, GPU hot path) vs the reference's invert."""
    from sgl_analytic_gb300 import generate_pdf_lnmu
    from tests.conftest import GOLDEN
    x = ref_sub["xi_out"]
    xo, p, info = generate_pdf_lnmu(1.0, lnmu=x, population=GOLDEN / "pop_zs1_sub.npz", return_info=True)
    np.testing.assert_array_equal(xo, x)
    dpeak, l1, _ = _pdf_errors(p, ref_sub["pdfx_P"], x)
    assert dpeak <= TOL_PEAK
    assert info["grid"]["nk_k"] == int(ref_sub["pdfx_grid"][0])
    assert {"diagnostics", "moment_interval", "t_stages", "sigma_kappa"} <= set(info)


def test_cli_end_to_end(tmp_path, ref_sub):
    import json as _json
    from sgl_analytic_gb300 import cli
    from tests.conftest import GOLDEN
    dest = tmp_path / "pdf.json"
    cli.main(["--z-s", "1", "--population", str(GOLDEN / "pop_zs1_sub.npz"), "--out", str(dest)])
    d = _json.loads(dest.read_text())
    P = np.array(d["P_s"] + d["P_s_tail"])
    dpeak, _, _ = _pdf_errors(P, ref_sub["pdfx_P"], ref_sub["xi_out"])
    assert dpeak <= TOL_PEAK
    # the reference's output keys: pipeline.run's dict (pipeline.py:243-271) and the CLI's additions
    # (cli.py:65-70)
    run_keys = {"t_stages", "zs", "cfg", "zint", "zint_n", "clustering", "xi_kperp", "edge", "lss_var", "kap_floor",
                "kbar", "h", "Om", "s8", "Ob", "ns", "zeq", "sigma8", "Ok", "w0", "wa", "growth_mode", "radiation",
                "Omega_r", "nord", "grid_scale", "split", "nproc", "sub_kw", "pair_angle", "k3", "exactS", "s_taper",
                "sigma_kappa", "kthr", "N_expl", "N_fil", "V_weak", "mean", "var", "skew", "sigmaDL", "grid",
                "tail_box", "fine", "s_is", "xi_closure", "window", "n_xi_wide", "pos_closure",
                "direct_product_backend", "s_seed", "s_seed_effective", "s_ess", "is_design", "seconds", "xi", "P_s",
                "xi_tail", "P_s_tail"}
    cli_keys = {"moment_interval", "diagnostics", "clipped"}
    assert run_keys | cli_keys <= set(d), sorted(run_keys | cli_keys - set(d))
    assert d["window"] is False and d["n_xi_wide"] == 500 and d["xi_closure"] == "gauss"
    assert {"nk_k", "nk_g", "n_kap", "n_gam", "xi_min", "xi_max"} <= set(d["grid"])
    assert {"grid_mass", "negative_mass", "minimum_density"} == set(d["diagnostics"])
    assert {"mean", "var", "skew"} == set(d["clipped"])


def test_xi_preparation_paths_agree(pop_sub, monkeypatch):
    """The xi groups prepared on the GPU from the caller's rows (coherent host access) and on the
    host give the same ln Phi and PDF (summation orders differ: ~1e-15 relative)."""
    from sgl_analytic_gb300 import Lam, invert
    kk, kg = KK16, KG_FULL
    a = Lam(pop_sub, xi=True)
    La = a(kk, kg)
    monkeypatch.setenv("SGL_XI_HOST_PREP", "1")
    b = Lam(pop_sub, xi=True)
    Lb = b(kk, kg)
    assert a.sigma() == pytest.approx(b.sigma(), rel=1e-14)
    assert np.max(np.abs(La - Lb)) <= 1e-12 * max(1.0, np.max(np.abs(La)))
    x = np.linspace(-0.35, 0.55, 200)
    Pa = invert(a, a.sigma(), xi_out=x, phi_tol=1e-8)[1]
    Pb = invert(b, b.sigma(), xi_out=x, phi_tol=1e-8)[1]
    assert np.max(np.abs(Pa - Pb)) <= 1e-12 * np.max(Pa)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_grid_above_block_threshold_matches_reference(precision):
    """A 5267 x 5282 = 2.78e7-point k-grid, where the reference inverts in k_kappa row blocks
    (_invert_blocked, sgl_full.py:97-157): the same sums, unblocked in HBM, against the reference's
    own output on that case (tests/golden/make_blocked_golden.py)."""
    from sgl_analytic_gb300 import Lam, Population, invert
    ref = dict(np.load(GOLDEN / "ref_blocked.npz"))
    lam = Lam(Population.load(GOLDEN / "pop_blocked.npz"), xi=False)
    assert lam.sigma() == pytest.approx(float(ref["sigma"]), rel=1e-12)
    x = ref["xi_out"]
    _, P, meta = invert(lam, lam.sigma(), xi_out=x, phi_tol=1e-8, precision=precision)
    g = meta["grid"]
    assert [g["nk_k"], g["nk_g"], g["n_kap"], g["n_gam"]] == [int(v) for v in ref["grid"][[0, 1, 4, 5]]]
    assert g["nk_k"] * g["nk_g"] > 2e7
    dpeak, l1, rel_tail = _pdf_errors(P, ref["P"], x)
    if precision == "fp64":
        assert dpeak <= TOL_PEAK, dpeak
    else:
        # 300 cells carrying the weight of 80k: ln Phi is a sum of few large terms, and the worst
        # tail point sits at 1.0e-6 of the peak.  The mixed path evaluates ln Phi in FP64 for so
        # few cells (FP32 transforms): tail 7.6e-4 (1.2e-3 with FP32 ln Phi).
        assert l1 <= 1e-4, (dpeak, l1, rel_tail)
        assert rel_tail <= 1e-3, (dpeak, l1, rel_tail)


@pytest.mark.parametrize("zs", ["3", "10", "0.5"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_other_redshifts_match_stored_golden(zs, precision):
    """The reference's own z_s population (tests/golden/make_fixtures.py, all xi groups) through the
    whole GPU chain against the reference's stored PDF for that z_s (pdf_zs<z>.json)."""
    from sgl_analytic_gb300 import Lam, Population, invert
    from tests.conftest import FULL_DIR
    path = FULL_DIR / f"cells_zs{zs}_gauss_full.npz"
    if not path.exists():
        pytest.skip(f"full z_s={zs} population not present")
    lam = Lam(Population.load(path), xi=True)
    ref = json.load(open(GOLDEN / f"pdf_zs{zs}.json"))
    assert lam.sigma() == pytest.approx(ref["sigma_kappa"], rel=1e-9)
    x = np.concatenate([ref["xi"], ref["xi_tail"]])
    _, P, meta = invert(lam, lam.sigma(), xi_out=x, phi_tol=1e-8, precision=precision)
    P0 = np.concatenate([ref["P_s"], ref["P_s_tail"]])
    g, rg = meta["grid"], ref["grid"]
    assert [g[k] for k in ("nk_k", "nk_g", "n_kap", "n_gam")] == [rg[k] for k in ("nk_k", "nk_g", "n_kap", "n_gam")]
    dpeak, l1, rel_tail = _pdf_errors(P, P0, x)
    if precision == "fp64":
        assert dpeak <= TOL_PEAK, dpeak
    else:
        assert l1 <= 1e-4 and rel_tail <= 1e-3, (dpeak, l1, rel_tail)


def test_invert_caller_phi_matches_pdf_and_reference(lamx, ref_sub):
    """sgl_plan_grid + sgl_invert on Phi = exp(ln Phi) evaluated by the caller (here through sgl_lnphi)
    reproduce sgl_pdf and the reference's invert on the same population (FP64 bar)."""
    eng = lamx.engine
    x = ref_sub["xi_out"]
    g = eng.plan_grid(phi_tol=1e-8)
    assert [g["nk_k"], g["nk_g"], g["n_kap"], g["n_gam"]] == [int(v) for v in ref_sub["pdfx_grid"][[0, 1, 4, 5]]]
    kk = np.linspace(0.0, g["k_k_max"], g["nk_k"])
    kg = np.linspace(0.0, g["k_g_max"], g["nk_g"])
    phi = np.exp(lamx(kk, kg))
    P, meta = eng.invert_phi(phi, g, x, phi_tol=1e-8)
    P_pdf, _ = eng.pdf(x, phi_tol=1e-8)
    peak = np.max(P_pdf)
    assert np.max(np.abs(P - P_pdf)) <= 1e-12 * peak
    dpeak, l1, _ = _pdf_errors(P, ref_sub["pdfx_P"], x)
    assert dpeak <= TOL_PEAK
    assert meta["nk_k"] == g["nk_k"] and meta["window"] == 0.0
    # the same Phi from device memory, and the mixed path on it
    torch = pytest.importorskip("torch")
    re = torch.tensor(phi.real, dtype=torch.float64, device="cuda:0")
    im = torch.tensor(phi.imag, dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    Pd, _ = eng.invert_phi((re.data_ptr(), im.data_ptr()), g, x, phi_tol=1e-8)
    assert np.max(np.abs(Pd - P)) <= 1e-14 * peak
    from sgl_analytic_gb300._lib import SGL_MIXED
    Pm, _ = eng.invert_phi(phi, g, x, precision=SGL_MIXED, phi_tol=1e-8)
    _, l1m, tailm = _pdf_errors(Pm, ref_sub["pdfx_P"], x)
    assert l1m <= 1e-4 and tailm <= 1e-3, (l1m, tailm)


def test_invert_rejects_bad_grids(lamx):
    eng = lamx.engine
    g = eng.plan_grid(phi_tol=1e-8)
    phi = np.ones((g["nk_k"], g["nk_g"]), complex)
    with pytest.raises(ValueError):
        eng.invert_phi(phi[:, :-1], g, np.zeros(3))
    bad = dict(g, sigma=-1.0)
    with pytest.raises(ValueError):
        eng.invert_phi(phi, bad, np.zeros(3))
    bad = dict(g, nk_k=1, nk_g=g["nk_g"])
    with pytest.raises(ValueError):
        eng.invert_phi(np.ones((1, g["nk_g"]), complex), bad, np.zeros(3))


def test_native_batch_matches_single_context(pop_sub, ref_sub):
    """sgl_batch_*: PDFs on 3 slots from the batch's own host threads, jobs interleaved over the slots,
    equal the single-context sgl_pdf result (FP64: the same sums in the same order)."""
    from sgl_analytic_gb300 import Lam
    from sgl_analytic_gb300._lib import Batch
    x = ref_sub["xi_out"]
    b = Batch(3)
    try:
        for i in range(3):
            Lam(pop_sub, xi=True, engine=b.slot(i))
        P, metas = b.pdf([0, 1, 2, 0, 2], x, phi_tol=1e-8)
        assert P.shape == (5, x.size) and len(metas) == 5
        single, _ = Lam(pop_sub, xi=True).engine.pdf(x, phi_tol=1e-8)
        for row in P:
            np.testing.assert_array_equal(row, single)
        dpeak, _, _ = _pdf_errors(P[0], ref_sub["pdfx_P"], x)
        assert dpeak <= TOL_PEAK
        with pytest.raises(ValueError):
            b.pdf([0, 3], x)                       # no slot 3
    finally:
        b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_window_matches_reference(precision):
    """The positive-definite box window (_window_pd, sgl_full.py:83-94, 254-258) against the reference's
    invert(window=True) on a 1000-cell population (tests/golden/make_window_golden.py); the same
    population without the window as well, so the window's effect is what is checked."""
    from sgl_analytic_gb300 import Lam, Population, invert
    ref = dict(np.load(GOLDEN / "ref_window.npz"))
    lam = Lam(Population.load(GOLDEN / "pop_window.npz"), xi=False)
    assert lam.sigma() == pytest.approx(float(ref["sigma"]), rel=1e-12)
    x = ref["xi_out"]
    effect = np.max(np.abs(ref["win_P"] - ref["raw_P"])) / np.max(ref["raw_P"])
    assert effect > 1e-3                                  # the window changes this PDF
    for tag, win in (("win", True), ("raw", False)):
        _, P, meta = invert(lam, lam.sigma(), xi_out=x, phi_tol=1e-8, window=win, precision=precision)
        g = meta["grid"]
        assert [g["nk_k"], g["nk_g"], g["n_kap"], g["n_gam"]] == [int(v) for v in ref[tag + "_grid"][[0, 1, 4, 5]]]
        assert g["window"] == float(ref[tag + "_grid"][11])
        dpeak, l1, rel_tail = _pdf_errors(P, ref[tag + "_P"], x)
        if precision == "fp64":
            assert dpeak <= TOL_PEAK, (tag, dpeak)
        else:
            assert l1 <= 1e-4 and dpeak <= 1e-5, (tag, dpeak, l1)
