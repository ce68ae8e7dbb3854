"""The GPU cell deposit (sgl_cells_*, sgl_analytic_gb300.cells.Cells) against the reference's own Cells
outputs (tests/golden/make_cells_golden.py) and the oracle."""
import numpy as np
import pytest

from tests import cells_replay as CR

pytestmark = pytest.mark.gpu

# FP64 atomics add each bin's terms in another order than the reference's loop: positive terms agree to
# a few ulps per term; a group's rows go through a Gram matrix and its eigenvectors (Jacobi here, LAPACK
# there)
RTOL_BINS = 1e-12
TOL_ROWS = 1e-9


@pytest.fixture(scope="module")
def gold():
    return CR.load()


def _check_bins(c, gold, tag):
    for name in ("H0", "H0k", "H0g", "Hc"):
        got = np.asarray(getattr(c, name))
        want = CR.dense(gold, tag, name, got.shape)
        assert np.array_equal(got != 0, want != 0), name
        # H0k's central bin (-1e-7, 1e-7) holds kappa of both signs: its sum may cancel
        np.testing.assert_allclose(got, want, rtol=RTOL_BINS, atol=1e-14 * np.abs(want).max(), err_msg=name)
    N = float(gold[f"{tag}_N"])
    assert c.N == pytest.approx(N, rel=1e-13)
    assert c.dropped == pytest.approx(float(gold[f"{tag}_dropped"]), abs=1e-13 * N)
    keys = [tuple(k) for k in gold[f"{tag}_lin_keys"]]
    assert sorted((int(s), b) for s, b in c.lin) == sorted((int(s), b) for s, b in keys)
    for (s, b), v in zip(keys, gold[f"{tag}_lin_vals"]):
        assert c.lin[(int(s), b)] == pytest.approx(v, rel=1e-12, abs=1e-13 * N)


def test_deposit_matches_reference(gold):
    from sgl_analytic_gb300.cells import Cells
    c = CR.replay(Cells(3, 3), gold, "plain")
    _check_bins(c, gold, "plain")


def test_batched_deposit_matches_reference(gold):
    """All 30 objects in one call: the same lattices and per-object totals."""
    from sgl_analytic_gb300.cells import Cells
    c = CR.replay(Cells(3, 3), gold, "plain", batched=True)
    _check_bins(c, gold, "plain")


def test_xi_node_matches_reference(gold):
    from sgl_analytic_gb300.cells import Cells
    c = CR.replay(Cells(2, 3, xi=CR.xi_dict(gold)), gold, "xi")
    _check_bins(c, gold, "xi")
    CR.check_groups(c.xi_groups, gold, "xi", tol=TOL_ROWS, rtol_w=RTOL_BINS)


def test_xi_node_batched_matches_oracle(gold):
    from oracle.cells_oracle import CellsOracle
    from sgl_analytic_gb300.cells import Cells
    c = CR.replay(Cells(2, 3, xi=CR.xi_dict(gold)), gold, "xi", batched=True)
    o = CR.replay(CellsOracle(2, 3, xi=CR.xi_dict(gold)), gold, "xi")
    assert len(c.xi_groups) == len(o.xi_groups)
    for g, h in zip(c.xi_groups, o.xi_groups):
        assert g["m"] == h["m"] and np.array_equal(g["idx"], h["idx"])
        f = np.random.default_rng(5).standard_normal((g["idx"].size + 1, 4))
        Pg, Ph = g["rows"].T @ (g["rows"] @ f), h["rows"].T @ (h["rows"] @ f)
        s0 = np.linalg.norm(h["rows"], axis=1).max()
        np.testing.assert_allclose(Pg, Ph, rtol=0, atol=TOL_ROWS * s0 ** 2 * np.abs(f).max() * 4)


def test_population_from_gpu_cells(gold):
    """Population.from_cells reads a GPU build as it reads the reference's."""
    from oracle.cells_oracle import CellsOracle
    from sgl_analytic_gb300.cells import Cells
    from sgl_analytic_gb300.population import Population
    c = CR.replay(Cells(2, 3, xi=CR.xi_dict(gold)), gold, "xi")
    o = CR.replay(CellsOracle(2, 3, xi=CR.xi_dict(gold)), gold, "xi")
    P, Q = Population.from_cells(c), Population.from_cells(o)
    assert np.array_equal(P.ig, Q.ig)
    np.testing.assert_allclose(P.w0, Q.w0, rtol=1e-12)
    np.testing.assert_allclose(P.k0, Q.k0, rtol=1e-11, atol=1e-18)
    np.testing.assert_allclose(P.g0, Q.g0, rtol=1e-11)
    assert np.array_equal(P.xg_m, Q.xg_m) and np.array_equal(P.xg_idx, Q.xg_idx)


def test_edge_cases_and_errors():
    from sgl_analytic_gb300.cells import Cells, FINE
    c = Cells(2, 2)
    hi = FINE["k"][1]
    # the last edges go into the last bins, NaN and out-of-lattice points are dropped but counted
    K = np.array([hi, -hi, 0.0, np.nan, 1.0, 2 * hi, 1e-3])
    G = np.array([hi, 1e-3, 0.0, 1e-3, np.nan, 1e-3, 1e-20])
    W = np.array([1.0, 2.0, 4.0, 8.0, 16.0, 32.0, 64.0])
    c.add(K, G, W, 1, 0.5)
    c.add(np.zeros(0), np.zeros(0), np.zeros(0), 0, 1.0)        # empty object
    from oracle.cells_oracle import CellsOracle
    o = CellsOracle(2, 2)
    o.add(K, G, W, 1, 0.5)
    o.add(np.zeros(0), np.zeros(0), np.zeros(0), 0, 1.0)
    for name in ("H0", "H0k", "H0g", "Hc"):
        assert np.array_equal(getattr(c, name), getattr(o, name)), name
    assert c.N == o.N and c.dropped == o.dropped and c.lin == o.lin
    with pytest.raises(ValueError):
        c.add(K, G, W, 2, 1.0)                                   # shell out of range
    with pytest.raises(ValueError):
        c.add(K, G, W, 0, np.inf)
    with pytest.raises(ValueError):
        c.add(K, G[:3], W, 0, 1.0)
    x = Cells(1, 1, xi=dict(kp=np.array([0.1, 1.0]), c=np.array([1.0, 1.0]), mmax=2))
    with pytest.raises(RuntimeError):
        x.add(K, G, W, 0, 1.0, R=np.ones(K.size))                # outside xi_begin / xi_end
    x.xi_begin(10.0)
    with pytest.raises(NotImplementedError):
        x.add(K, G, W, 0, 1.0)                                   # no lens distances


def test_real_shell_matches_reference():
    """Every deposit of one lens shell of the reference's own z_s = 1 build (hosts, filaments, the exact
    subhalo sector, xi_lin nodes; recorded by tests/golden/make_cells_golden.py shell) replayed into the
    GPU deposit, against that shell's Cells outputs."""
    from sgl_analytic_gb300.cells import Cells
    d = CR.shell_record()
    if d is None:
        pytest.skip("recorded shell not present")
    c = Cells(1, int(d["nord"]), xi=dict(kp=d["xi_kp"], c=d["xi_c"], mmax=int(d["xi_mmax"])))
    CR.check_shell(CR.replay_shell(c, d), d, RTOL_BINS, TOL_ROWS)


def test_lattice_attributes_are_stable_arrays():
    """The reference's build merges per-shell pieces into a result Cells by editing H0 / Hc in place
    (sgl_full.py:1790-1797) and reads them back later: the arrays returned stay the same objects until
    the next deposit."""
    from sgl_analytic_gb300.cells import Cells
    c = Cells(2, 1)
    h = c.H0
    h.reshape(-1)[[3, 7]] += [1.5, 2.5]
    c.Hc[1] += 1.0
    assert c.H0 is h and c.H0.reshape(-1)[7] == 2.5 and np.all(c.Hc[1] == 1.0)
    c.add(np.array([0.5]), np.array([0.5]), np.array([1.0]), 0, 1.0)
    assert c.H0.reshape(-1)[7] == 0.0 and c.H0.sum() == 1.0     # a deposit reads the device lattices again
