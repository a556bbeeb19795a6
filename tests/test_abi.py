"""The C-ABI library: loads, exports every symbol include/tdz.h declares, and
its host-only entry points (space set-up, quadrature, error reporting) agree
with the oracle. No GPU work here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import bspline as ob

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from tdsez_gb300 import _lib, build
    build.build()
    return _lib.load()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "tdz.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tdz_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    from tdsez_gb300 import _lib
    names = declared_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_space_quadrature_matches_oracle(lib):
    from tdsez_gb300.space import Space
    kn = ob.interface_knots(-15.0, 15.0, 11, 3, [-6.0, 3.0])
    S = Space([kn], 3, 4)
    ax = ob.Axis(kn, 3, 4)
    assert S.n[0] == ax.n and S.nel[0] == ax.nel
    x, w = S.quadrature(0)
    assert np.abs(x - ax.xq.reshape(-1)).max() < 1e-14
    assert np.abs(w - ax.wq.reshape(-1)).max() < 1e-14


def test_knot_generators_match_oracle():
    from tdsez_gb300 import space as ps
    assert np.array_equal(ps.uniform_knots(9, -3.0, 4.0, 4), ob.uniform_knots(9, -3.0, 4.0, 4))
    assert np.array_equal(ps.symexp_knots(-60, 60, 32, 0.9, 4), ob.symexp_knots(-60, 60, 31, 0.9, 4))
    assert np.array_equal(ps.interface_knots(-15, 15, 12, 3, [-6, 3]), ob.interface_knots(-15, 15, 11, 3, [-6, 3]))


def test_errors_are_status_codes(lib):
    h = C.c_void_p()
    k = (C.c_double * 3)(0.0, 0.5, 1.0)
    arr = (C.POINTER(C.c_double) * 1)(C.cast(k, C.POINTER(C.c_double)))
    st = lib.tdz_space_create(1, (C.c_int * 1)(3), (C.c_int * 1)(3), arr, 4, C.byref(h))
    assert st == 1  # TDZ_ERR_ARG: too few knots
    assert b"too few knots" in lib.tdz_last_error()
    st = lib.tdz_space_create(4, None, None, None, 4, C.byref(h))
    assert st == 1
    assert lib.tdz_version().startswith(b"tdz")
