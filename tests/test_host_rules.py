"""Host-only rules of the propagation path, through the C ABI against the
oracle's restatements (no GPU work): the preconditioner refresh rule of
TDSEZPCRefresh (include/tdsez_propagator.hpp:17-31) and the strong-field
check of TDSEZSetupMultigrid (src/multigrid.cpp:213-237)."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle.propagate import PCRefreshRule, strong_field_ratio


@pytest.fixture(scope="module")
def lib():
    from tdsez_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.mark.parametrize("cap", [-1, 0, 7, 12])
def test_pc_refresh_rule_matches_reference_rule(lib, cap):
    """Synthetic iteration counts: steady, slowly growing, jumps past
    2 base + 5, jumps past the cap, and a rebuilt base."""
    from tdsez_gb300 import _lib
    rng = np.random.default_rng(20261203)
    its = [4, 4, 5, 13, 14, 3, 3, 11, 12, 30, 2, 9, 10, 0, 6, 17, 8, 8]
    its += list(rng.integers(0, 40, 200))
    st = _lib.tdz_pc_refresh(base=-1, rebuilds=0, cap=cap)
    ref = PCRefreshRule(cap)
    for k in its:
        got = lib.tdz_pc_refresh_stale(C.byref(st), int(k))
        want = ref.stale(int(k))
        assert bool(got) == want, (cap, k)
        assert (st.base, st.rebuilds) == (ref.base, ref.rebuilds)
    assert ref.rebuilds > 0


def test_pc_refresh_rule_cases(lib):
    """The rule's two triggers, by hand: base 4 -> rebuild above 13; cap 10."""
    from tdsez_gb300 import _lib
    st = _lib.tdz_pc_refresh(base=-1, rebuilds=0, cap=-1)
    seq = [(4, 0), (13, 0), (14, 1), (20, 0), (45, 0), (46, 1)]
    for its, want in seq:
        assert lib.tdz_pc_refresh_stale(C.byref(st), its) == want, its
    st = _lib.tdz_pc_refresh(base=-1, rebuilds=0, cap=10)
    assert [lib.tdz_pc_refresh_stale(C.byref(st), k) for k in (3, 10, 11, 2, 11)] == [0, 0, 1, 0, 1]
    assert st.rebuilds == 2


@pytest.mark.parametrize("kind", ["cn", "pade22", "magnus4"])
def test_strong_field_ratio_matches_reference_check(lib, kind):
    from tdsez_gb300.propagator import KINDS
    from tdsez_gb300.space import Space, uniform_knots
    from tdsez_gb300 import _lib
    knots = [uniform_knots(8, -30.0, 20.0, 3), uniform_knots(6, -10.0, 12.0, 3), uniform_knots(5, -5.0, 5.0, 3)]
    S = Space(knots, 3, 4)
    T, w0 = 2 * 2 * math.pi / 0.057, 0.057
    E = [0.05, 0.0, 0.02]

    def field(a, t):
        return E[a] * math.sin(math.pi * t / T) ** 2 * math.cos(w0 * t)
    cb = _lib.FIELD_FN(lambda a, t, ctx: field(a, t))
    out = C.c_double()
    for dt in (0.05, 0.5):
        _lib.check(lib.tdz_strong_field_ratio(S.handle, KINDS[kind], dt, T, cb, None, C.byref(out)))
        want = strong_field_ratio(kind, dt, T, field, [(-30.0, 20.0), (-10.0, 12.0), (-5.0, 5.0)])
        assert abs(out.value - want) <= 1e-13 * want, (dt, out.value, want)


def test_strong_field_warning_from_evolve_needs_no_gpu_for_the_check(lib):
    """The ratio is computed on the host before any step: a strong field is
    flagged for the multigrid preconditioner (1D HO box [-20, 20], E0 = 0.5,
    CN dt = 0.5: tau max|E.r| = 0.25 * 0.5 * 20 = 2.5 > 1.5)."""
    from oracle.propagate import strong_field_ratio as ref
    T = 100.0
    r = ref("cn", 0.5, T, lambda a, t: 0.5 * math.sin(math.pi * t / T) ** 2, [(-20.0, 20.0)])
    assert r > 1.5
