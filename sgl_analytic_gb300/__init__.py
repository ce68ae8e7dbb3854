"""GB300 (sm_103a) engine for the hot path of sampling-free weak-lensing magnification PDFs.

Drop-in for the reference package ``sgl_analytic``'s characteristic-exponent / inversion path:
``Lam`` and ``invert`` (sgl_full.py), and through them ``generate_pdf_lnmu``, ``generate_pdf`` and
the CLI.  The arithmetic runs in hand-written CUDA kernels behind the C ABI of
``include/sgl_gb300.h``; there is no CPU fallback.
"""
from .lam import Lam, invert
from .population import Population

__version__ = "0.1.0"
__all__ = ["Lam", "invert", "Population", "generate_pdf", "generate_pdf_lnmu", "install", "__version__"]


def __getattr__(name):
    if name in ("generate_pdf", "generate_pdf_lnmu"):
        from . import api
        return getattr(api, name)
    if name == "install":
        from .plugin import install
        return install
    raise AttributeError(name)
