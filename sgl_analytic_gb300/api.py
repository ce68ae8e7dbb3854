"""Public API with the reference's signatures (sgl_analytic api.py:26-113).

Same parameter names, defaults, validation and errors; the hot path (Lam + invert) runs on the
GPU.  Extra keyword-only arguments: ``population`` (a pre-built ``Population`` or ``.npz``; else
the reference package builds it on the CPU), ``precision`` ("fp64" parity path or "mixed") and
``device``.
"""
import warnings

import numpy as np

from .pipeline import run


def _grid(values, lo, hi, count, name):
    """Grid validation of the reference (api.py:11-23)."""
    if values is None:
        if isinstance(count, bool) or not isinstance(count, (int, np.integer)) or count < 2:
            raise ValueError(f"n_{name} must be an integer >= 2")
        if not np.isfinite(lo) or not np.isfinite(hi) or lo >= hi:
            raise ValueError(f"{name}_min and {name}_max must be finite and increasing")
        values = np.linspace(lo, hi, count)
    values = np.asarray(values, dtype=float)
    if values.ndim != 1 or values.size < 2 or not np.all(np.isfinite(values)):
        raise ValueError(f"{name} must be a finite one-dimensional grid with >= 2 points")
    if np.any(np.diff(values) <= 0):
        raise ValueError(f"{name} must be strictly increasing")
    return values


def generate_pdf_lnmu(z_s, h=0.674, Om=0.315, sigma8=0.811, Ob=0.0493, ns=0.965, zeq=3402.0, lnmu=None, *, Ok=0.0,
                      w0=-1.0, wa=0.0, growth_mode="ode", radiation="engine", closure="gauss", lnmu_min=-1.0,
                      lnmu_max=9.0, n_lnmu=3201, config="full", nproc=1, return_info=False, population=None,
                      precision="fp64", device=0):
    """Return (lnmu, dP_S/dlnmu) as NumPy arrays (reference api.py:26-84)."""
    x = _grid(lnmu, lnmu_min, lnmu_max, n_lnmu, "lnmu")
    out, _ = run(z_s, config, cosmo=dict(h=h, Om=Om, sigma8=sigma8, Ob=Ob, ns=ns, zeq=zeq, Ok=Ok, w0=w0, wa=wa,
                                         growth_mode=growth_mode, radiation=radiation),
                 xi_out=x, nproc=nproc, xi_closure=closure, population=population, precision=precision,
                 device=device)
    p = np.asarray(out.pop("P_s"))
    out.pop("xi")
    if not np.all(np.isfinite(p)):
        raise RuntimeError("PDF inversion returned non-finite values")
    negative_mass = float(np.trapezoid(np.maximum(-p, 0), x))
    out["diagnostics"] = dict(grid_mass=float(np.trapezoid(p, x)), negative_mass=negative_mass,
                              minimum_density=float(p.min()))
    out["moment_interval"] = [out["grid"]["xi_min"], out["grid"]["xi_max"]]
    if negative_mass > 0:
        warnings.warn(f"PDF inversion has negative residuals (integrated mass {negative_mass:.3g}); inspect "
                      f"diagnostics before using tail probabilities.", RuntimeWarning, stacklevel=2)
    return (x, p, out) if return_info else (x, p)


def generate_pdf(z_s, h=0.674, Om=0.315, sigma8=0.811, Ob=0.0493, ns=0.965, zeq=3402.0, mu=None, *, Ok=0.0,
                 w0=-1.0, wa=0.0, growth_mode="ode", radiation="engine", closure="gauss", mu_min=0.3, mu_max=30.0,
                 n_mu=2000, config="full", nproc=1, return_info=False, population=None, precision="fp64",
                 device=0):
    """Return (mu, p_S(mu)) with p(mu) = (dP/dlnmu)/mu (reference api.py:87-113)."""
    if mu is None:
        if mu_min <= 0 or mu_max <= 0:
            raise ValueError("mu bounds must be positive")
        x = _grid(None, np.log(mu_min), np.log(mu_max), n_mu, "mu")
        mu = np.exp(x)
    else:
        mu = _grid(mu, 0, 1, n_mu, "mu")
        if np.any(mu <= 0):
            raise ValueError("mu must be positive")
        x = np.log(mu)
    result = generate_pdf_lnmu(z_s, h, Om, sigma8, Ob, ns, zeq, x, Ok=Ok, w0=w0, wa=wa, growth_mode=growth_mode,
                               radiation=radiation, closure=closure, config=config, nproc=nproc,
                               return_info=return_info, population=population, precision=precision, device=device)
    return (mu, result[1] / mu, result[2]) if return_info else (mu, result[1] / mu)
