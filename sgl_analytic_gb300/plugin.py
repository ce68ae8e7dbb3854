"""Plugin route: run the reference package's own pipeline with this engine on its hot path.

``install()`` replaces ``sgl_analytic.sgl_full.Lam`` and ``sgl_analytic.sgl_full.invert`` -- the
two names the reference's ``pipeline.run`` calls for the hot path (pipeline.py:201, 237) -- with
the GPU versions, so that ``sgl_analytic.generate_pdf_lnmu``, ``generate_pdf`` and its CLI keep
their own population build and output assembly and hand the characteristic exponent and the
inversion to the GPU.  Configurations outside the GPU path raise ``NotImplementedError``.
``uninstall()`` restores the originals.
"""
from __future__ import annotations

_saved = {}


def install(precision="fp64", device=0, module=None):
    """Patch the reference's sgl_full module (or ``module``, for tests) in place."""
    if module is None:
        from sgl_analytic import sgl_full as module
    from .lam import Lam, invert
    if id(module) in _saved:
        return module
    _saved[id(module)] = (module.Lam, module.invert)

    class GpuLam(Lam):
        def __init__(self, cells, *args, **kw):
            kw.setdefault("precision", precision)
            kw.setdefault("device", device)
            super().__init__(cells, *args, **kw)

    def gpu_invert(lam, sigma, *args, **kw):
        return invert(lam, sigma, *args, **kw)

    module.Lam = GpuLam
    module.invert = gpu_invert
    return module


def uninstall(module=None):
    if module is None:
        from sgl_analytic import sgl_full as module
    if id(module) in _saved:
        module.Lam, module.invert = _saved.pop(id(module))
