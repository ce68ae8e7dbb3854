"""The GPU cosmology tables (sgl_cosmo_tables) against the reference's own chain Cosmology
(tests/golden/cosmo_ref.npz, made by tests/golden/make_cosmo_golden.py from sgl.py)."""
import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tables():
    from sgl_analytic_gb300._lib import Engine
    ref = dict(np.load(GOLDEN / "cosmo_ref.npz"))
    eng = Engine(0)
    return eng, ref, eng.cosmo_tables(ref["params"], ref["z"], ref["M"], ref["z_mf"])


def _rel(a, b):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def test_background_matches_reference(tables):
    _, ref, t = tables
    assert _rel(t["E"], ref["E"]) < 1e-14
    nz = ref["z"] > 0
    assert _rel(t["chi"][:, nz], ref["chi"][:, nz]) < 1e-12              # the reference's quad: ~1e-14
    assert _rel(t["DM"][:, nz], ref["DM"][:, nz]) < 1e-12
    assert np.all(t["chi"][:, ~nz] == 0)


def test_growth_matches_reference(tables):
    """Growth ODE: RK4 here, DOP853 at rtol 2e-10 in the reference."""
    _, ref, t = tables
    assert _rel(t["D"], ref["D"]) < 1e-9


def test_sigma_and_mass_function_match_reference(tables):
    _, ref, t = tables
    assert _rel(t["sigmaM"], ref["sigmaM"]) < 1e-9
    assert np.max(np.abs(t["dlnsig"] - ref["dlnsig"])) < 1e-9
    live = ref["dndlnM"] > 1e-300
    assert _rel(t["dndlnM"][live], ref["dndlnM"][live]) < 1e-7
    assert _rel(t["conc"], ref["conc"]) < 1e-9


def test_sigma_cr_matches_reference(tables):
    from sgl_analytic_gb300 import cosmology as CO
    eng, ref, _ = tables
    assert _rel(CO.sigma_cr(eng, ref["params"], ref["pairs"]), ref["Sigma_cr"]) < 1e-12


def test_domain_errors_are_the_references():
    from sgl_analytic_gb300._lib import Engine
    eng = Engine(0)
    base = [0.674, 0.315, 0.0493, 0.811, 0.965, 3402.0, 0.0, -1.0, 0.0]
    for k, v, msg in ((7, 0.5, "w0 + wa < 0"), (7, -2.5, "-2 <= w0"), (2, 0.4, "0 < Ob < Om"), (0, -1.0, "finite positive")):
        p = list(base)
        p[k] = v
        with pytest.raises(ValueError, match=msg.replace("+", r"\+")):
            eng.cosmo_tables(np.array([p]), [0.5], [1e12])
