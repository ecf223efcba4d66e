"""CPU checks of the C ABI: the library builds, loads, exports every symbol
declared in include/pisurf.h, carries the same DMC tables as the oracle, and
refuses to compute (PI_ERR_CUDA) where no GPU is present."""
import ctypes
import os
import re

import numpy as np
import pytest

from particleisosurface_gb300 import _native as N
from particleisosurface_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _lib():
    B.build()
    return N.lib()


def declared_symbols():
    h = open(os.path.join(ROOT, "include", "pisurf.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    return sorted(set(re.findall(r"\b(pi_[a-z0-9_]+)\s*\(", h)))


def test_exports_every_declared_symbol():
    syms = declared_symbols()
    assert len(syms) >= 25
    lib = ctypes.CDLL(N.LIB_PATH)
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_params_default_and_version():
    p = N.default_params(0.02)
    assert p.radius == pytest.approx(0.02) and p.smooth_factor == 2.0 and p.qef == 0
    assert b"sm_103a" in N.lib().pi_version()


def test_dmc_table_same_as_oracle():
    import pyoracle as O
    O.build()
    t1, f1, c1 = N.dmc_table()
    t2, f2, c2 = O.dmc_table()
    np.testing.assert_array_equal(t1, t2)
    np.testing.assert_array_equal(f1, f2)
    np.testing.assert_array_equal(c1, c2)


def test_no_cpu_fallback_without_gpu():
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    with pytest.raises(N.PiError) as e:
        N.Context(0)
    assert "PI_ERR_CUDA" in str(e.value) or "PI_ERR_INVALID" in str(e.value)


def test_null_arguments_rejected():
    h = ctypes.c_void_p()
    assert N.lib().pi_frame_create(None, None, ctypes.byref(h)) == -1
    assert N.lib().pi_frame_upload(None, None, 0) == -1
    assert N.lib().pi_run(None) == -1
    assert b"null" in N.lib().pi_last_error()
