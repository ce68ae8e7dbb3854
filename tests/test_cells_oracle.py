"""The deposit oracle (oracle/cells_oracle.py) against the reference's own Cells outputs
(tests/golden/make_cells_golden.py)."""
import numpy as np
import pytest

from tests import cells_replay as CR


@pytest.fixture(scope="module")
def gold():
    return CR.load()


def test_oracle_histograms_bit_exact(gold):
    from oracle.cells_oracle import CellsOracle
    c = CR.replay(CellsOracle(3, 3), gold, "plain")
    CR.check_histograms(c, gold, "plain", rtol=0)


def test_oracle_xi_build(gold):
    from oracle.cells_oracle import CellsOracle
    c = CR.replay(CellsOracle(2, 3, xi=CR.xi_dict(gold)), gold, "xi")
    CR.check_histograms(c, gold, "xi", rtol=0)
    # the reference's default sums a radius's points per bin before the k_perp loop: the same sums
    # in another order
    CR.check_groups(c.xi_groups, gold, "xi", tol=1e-10)


def test_oracle_bin_index_edges():
    from oracle.cells_oracle import FINE, bin_index, signed_log_edges
    e = signed_log_edges(FINE["k"])
    v = np.array([-np.inf, e[0], e[0] * (1 - 1e-16), e[1], 0.0, e[-1], np.nextafter(e[-1], 0), np.inf, np.nan])
    i = bin_index(v.copy(), e)
    assert i.tolist() == [0, 1, 1, 2, e.size // 2, e.size - 1, e.size - 1, e.size, e.size]


def test_oracle_real_shell():
    """The oracle on one real shell of the reference's z_s = 1 build: histograms bit for bit."""
    from oracle.cells_oracle import CellsOracle
    d = CR.shell_record()
    if d is None:
        pytest.skip("recorded shell not present")
    c = CellsOracle(1, int(d["nord"]), xi=dict(kp=d["xi_kp"], c=d["xi_c"], mmax=int(d["xi_mmax"])))
    CR.check_shell(CR.replay_shell(c, d), d, 0.0, 1e-10, exact=True)


def test_deposit_bench_workload_shape():
    """The bench's deposit node: 2048 hosts of 12 x 260 cells and 512 filaments of 120 x 12, each
    object's arrays aligned, weights positive, lens distances positive, filaments untangential."""
    from sgl_analytic_gb300.workloads import deposit_node
    objs, dchi = deposit_node(seed=0, n_host=8, n_fil=4)
    assert dchi > 0 and len(objs) == 12
    for o in objs[:8]:
        assert o["K"].size == o["G"].size == o["W"].size == o["R"].size == 12 * 260 and o["tang"]
    for o in objs[8:]:
        assert o["K"].size == 120 * 12 and not o["tang"]
    for o in objs:
        assert np.all(o["W"] >= 0) and np.all(o["R"] > 0) and np.all(np.isfinite(o["K"]))
    full, _ = deposit_node(seed=0)
    assert sum(o["K"].size for o in full) == 2048 * 3120 + 512 * 1440
