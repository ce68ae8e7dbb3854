"""Public input contracts of the drop-in API, without GPU solves (mirrors the reference's
tests/test_api.py contracts: validation before any solve, forwarding, the mu Jacobian, the
negative-residual warning) plus the GPU-path limits, the plugin and the CLI."""
import json
from pathlib import Path
import types
from unittest.mock import patch

import numpy as np
import pytest

from sgl_analytic_gb300 import api, cli, pipeline, plugin
from sgl_analytic_gb300.api import generate_pdf, generate_pdf_lnmu
from sgl_analytic_gb300.pipeline import cosmology_params, on, run
from sgl_analytic_gb300.population import Population


@pytest.mark.parametrize("cfg", ["", "garbage", "+typo", "-typo"])
def test_invalid_configuration(cfg):
    with pytest.raises(ValueError):
        on(cfg)


def test_configurations():
    assert on("full") == {"ell", "fil", "sub", "bias"} and on("halo") == set()
    assert on("-sub") == {"ell", "fil", "bias"} and on("+ell") == {"ell"}


def test_invalid_grid_fails_before_solver():
    with patch("sgl_analytic_gb300.api.run") as solver:
        for grid in ([0, 0], [1, 0], [0, np.nan], [[0, 1]], [0]):
            with pytest.raises(ValueError):
                generate_pdf_lnmu(1, lnmu=grid)
        with pytest.raises(ValueError):
            generate_pdf(1, mu=[0, 1])
        solver.assert_not_called()


@pytest.mark.parametrize("cp", [dict(h=0), dict(Om=np.nan), dict(Ob=0.4), dict(zeq=-1), dict(sigma8=.8, s8=.8),
                                dict(Ok=np.nan), dict(Ok=True), dict(w0=0.0), dict(wa=np.inf), dict(wa=1.2),
                                dict(w0=-.5, wa=.45), dict(growth_mode="exact"), dict(Ok=-1.5),
                                dict(w0=-.9, growth_mode="legacy"), dict(radiation="yes"), dict(foo=1)])
def test_cosmology_validation(cp):
    with pytest.raises(ValueError):
        cosmology_params(cp)


def test_cosmology_defaults_and_extensions():
    c = cosmology_params(dict(Ok=-.05, w0=-1.1, wa=.2))
    assert (c["Ok"], c["w0"], c["wa"], c["growth_mode"], c["radiation"]) == (-.05, -1.1, .2, "ode", "engine")
    assert cosmology_params(dict(radiation="none"))["radiation"] is None
    assert cosmology_params(None)["s8"] == 0.811


def test_invalid_redshift_and_workers_fail_before_solve():
    with patch("sgl_analytic_gb300.lam.Lam") as lam:
        for zs in (0, -1, np.nan, np.inf):
            with pytest.raises(ValueError):
                run(zs, "full")
        for nproc in (0, -1, 1.5, True):
            with pytest.raises(ValueError):
                run(1, "full", nproc=nproc)
        for kw in (dict(edge="r500"), dict(xi_closure="lognormal"), dict(xi_closure="vp", clustering="linear"),
                   dict(edge="kthr")):
            with pytest.raises(ValueError):
                run(1, "full", **kw)
        with pytest.raises(ValueError):
            run(1, "-bias", xi_closure="vp")
        lam.assert_not_called()


def test_configurations_outside_the_gpu_path_raise(pop_sub):
    with patch("sgl_analytic_gb300.lam.Lam") as lam:
        with pytest.raises(ValueError):             # the vp closure needs a population that carries it
            run(1, "full", xi_closure="vp", population=pop_sub)
        with pytest.raises(NotImplementedError):
            run(1, "full", clustering="limber")
        lam.assert_not_called()
    from sgl_analytic_gb300.lam import Lam
    for kw in (dict(C=np.eye(2)), dict(exactS=True), dict(lss_var=1e-3), dict(lam_coarse=51), dict(xi_clamp=True)):
        with pytest.raises(NotImplementedError):
            Lam(None, **kw)


def test_parameter_forwarding_and_jacobian():
    def fake_run(zs, cfg, **kw):
        assert zs == 2
        assert kw["cosmo"] == dict(h=.7, Om=.3, sigma8=.9, Ob=.05, ns=.97, zeq=3450, Ok=0.0, w0=-1.0, wa=0.0,
                                   growth_mode="ode", radiation="engine")
        assert kw["xi_closure"] == "gauss" and kw["precision"] == "mixed"
        x = kw["xi_out"]
        return dict(xi=x.tolist(), P_s=np.ones_like(x).tolist(), grid=dict(xi_min=-.5, xi_max=2)), {}
    mu = np.array([.5, 1, 2])
    with patch("sgl_analytic_gb300.api.run", side_effect=fake_run):
        x, p, info = generate_pdf(2, .7, .3, .9, .05, .97, 3450, mu=mu, return_info=True, precision="mixed")
    np.testing.assert_array_equal(x, mu)
    np.testing.assert_array_equal(p, 1 / mu)
    assert info["moment_interval"] == [-.5, 2]


def test_negative_residual_is_visible():
    output = dict(xi=[0, 1], P_s=[-.1, 1], grid=dict(xi_min=0, xi_max=1))
    with patch("sgl_analytic_gb300.api.run", return_value=(output, {})):
        with pytest.warns(RuntimeWarning):
            _, p, info = generate_pdf_lnmu(1, lnmu=[0, 1], return_info=True)
    assert p[0] == -.1
    assert info["diagnostics"]["negative_mass"] == pytest.approx(.05)


def test_non_finite_output_raises():
    output = dict(xi=[0, 1], P_s=[np.nan, 1], grid=dict(xi_min=0, xi_max=1))
    with patch("sgl_analytic_gb300.api.run", return_value=(output, {})):
        with pytest.raises(RuntimeError):
            generate_pdf_lnmu(1, lnmu=[0, 1])


def test_plugin_install_and_uninstall():
    fake = types.SimpleNamespace(Lam=object, invert=len)
    mod = plugin.install(precision="mixed", module=fake)
    assert mod.Lam is not object and issubclass(mod.Lam, __import__("sgl_analytic_gb300").Lam)
    assert mod.invert is not len
    plugin.uninstall(module=fake)
    assert fake.Lam is object and fake.invert is len


def test_cli_writes_reference_schema(tmp_path):
    def fake_run(zs, cfg, **kw):
        x, t = kw["xi_out"], kw["xi_tail"]
        return dict(xi=x.tolist(), P_s=np.exp(-x ** 2).tolist(), xi_tail=t.tolist(), P_s_tail=(0 * t).tolist(),
                    grid=dict(xi_min=-1, xi_max=9), sigma_kappa=0.036, seconds=0.1), {}
    dest = tmp_path / "pdf.json"
    with patch("sgl_analytic_gb300.cli.run", side_effect=fake_run):
        cli.main(["--z-s", "1", "--out", str(dest), "--precision", "mixed"])
    d = json.loads(dest.read_text())
    assert len(d["xi"]) == 1601 and len(d["xi_tail"]) == 1600
    for key in ("moment_interval", "diagnostics", "clipped"):
        assert key in d


def test_population_from_cells_compaction():
    """Lam.__init__'s cell compaction: occupied bins, weight-averaged centroids (sgl_full.py:2759-2775)."""
    H0 = np.zeros((4, 3)); H0[1, 2] = 2.0; H0[3, 0] = 4.0
    cells = types.SimpleNamespace(H0=H0, H0k=H0 * 0.5, H0g=H0 * 0.25, wV=np.zeros((2, 2)),
                                  fe=[np.linspace(-1, 1, 5), np.geomspace(1e-9, 30, 4)], xi_groups=[])
    pop = Population.from_cells(cells)
    np.testing.assert_array_equal(pop.w0, [2.0, 4.0])
    np.testing.assert_array_equal(pop.k0, [0.5, 0.5])
    np.testing.assert_array_equal(pop.g0, [0.25, 0.25])
    np.testing.assert_array_equal(pop.ig, [2, 0])
    assert not pop.has_xi


def test_population_roundtrip(tmp_path, pop_sub):
    p = tmp_path / "pop.npz"
    pop_sub.save(p)
    back = Population.load(p)
    np.testing.assert_array_equal(back.w0, pop_sub.w0)
    assert back.xg_m.tolist() == pop_sub.xg_m.tolist()
    g = back.groups()
    assert len(g) == 3 and g[0]["rows"].shape == (int(back.xg_nrow[0]), int(back.xg_nidx[0]) + 1)
    sub = Population.load(p, groups=[1])
    assert sub.xg_m.tolist() == [1] and sub.xg_s0 > 0


def test_population_carries_the_vp_closure(tmp_path, pop_sub):
    """A population saved with its vp closure loads it back (Lam.install_vp's arrays)."""
    from dataclasses import replace
    vp = dict(np.load(Path(__file__).resolve().parent / "golden" / "vp_zs1_sub.npz"))
    vp = {k: vp[k] for k in Population.VP_FILE_KEYS if k in vp}
    pop = replace(pop_sub, vp=vp)
    p = tmp_path / "pop_vp.npz"
    pop.save(p)
    back = Population.load(p)
    assert set(back.vp) == set(vp)
    for k in vp:
        np.testing.assert_array_equal(back.vp[k], vp[k])
    assert Population.load(tmp_path / "pop_vp.npz").vp is not None
