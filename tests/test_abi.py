"""CPU checks of the C ABI: the library loads and exports every symbol the header declares.
No compute call is made (there is no GPU here)."""
import ctypes
import re

import pytest

from sgl_analytic_gb300 import _lib
from tests.conftest import ROOT

HEADER = ROOT / "include" / "sgl_gb300.h"


def declared():
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return set(re.findall(r"\b(sgl_[A-Za-z_0-9]+)\s*\(", txt))


def test_header_and_binding_agree():
    assert declared() == set(_lib.EXPORTS)


@pytest.mark.skipif(not _lib.LIB_PATH.exists(), reason="engine not built")
def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(str(_lib.LIB_PATH))
    for name in declared():
        assert hasattr(L, name), name
    assert L.sgl_abi_version() == 2


@pytest.mark.skipif(not _lib.LIB_PATH.exists(), reason="engine not built")
def test_defaults_and_error_buffer_without_gpu():
    L = _lib.lib()
    o = _lib.InvertOpts()
    L.sgl_invert_opts_default(ctypes.byref(o))
    assert (o.precision, o.tail_box, o.phi_tol, o.n_xi_wide, o.n_k_int, o.xi_reach, o.window) == \
        (0, 1, 1e-8, 500, 2400, 24.0, 0)
    buf = ctypes.create_string_buffer(64)
    assert L.sgl_last_error(None, buf, 64) >= 0
