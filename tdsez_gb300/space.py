"""Host side of the B-spline space: knot sequences and the tdz_space handle.

Knot generators mirror TDSE-Z's (the knots are inputs of the hot path):
``uniform`` (PetIGA ``IGAAxisInitUniform`` with C = p-1, ``src/core.cpp:1946``),
``symexp`` (``TDSEZExpSymKnots``, ``src/core_knots.cpp:77-120``) and
``interface`` (``TDSEZInterfaceKnots``, ``src/core_knots.cpp:318-385``).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Sequence

import numpy as np

from . import _lib


def uniform_knots(nel: int, lo: float, hi: float, p: int) -> np.ndarray:
    inner = [lo + (hi - lo) * i / nel for i in range(1, nel)]
    return np.array([lo] * (p + 1) + inner + [hi] * (p + 1), dtype=np.float64)


def symexp_knots(lo: float, hi: float, nel: int, alpha: float, p: int) -> np.ndarray:
    """nel elements (ninterior = nel - 1 graded interior knots)."""
    nint = nel - 1
    k = [lo] * (p + 1)
    for i in range(nint):
        t = 2.0 * (i + 1.0) / (nint + 1) - 1.0
        m = (math.exp(alpha * abs(t)) - 1.0) / (math.exp(alpha) - 1.0)
        k.append(m * hi if t >= 0.0 else m * lo)
    return np.array(k + [hi] * (p + 1), dtype=np.float64)


def interface_knots(lo: float, hi: float, nel: int, p: int, breakpoints: Sequence[float]) -> np.ndarray:
    """nel elements over the layers between breakpoints (largest remainder,
    at least one per layer), multiplicity p at every interface."""
    tol = 1e-9 * (hi - lo)
    brk = [lo]
    for x in sorted(breakpoints):
        if lo + tol < x < hi - tol and x > brk[-1] + tol:
            brk.append(x)
    brk.append(hi)
    nseg = len(brk) - 1
    if nel < nseg:
        raise ValueError("fewer elements than material segments")
    share = [nel * (brk[s + 1] - brk[s]) / (hi - lo) for s in range(nseg)]
    cnt = [max(1, int(math.floor(v))) for v in share]
    rem = [v - math.floor(v) for v in share]
    while sum(cnt) < nel:
        s = int(np.argmax(rem))
        cnt[s] += 1
        rem[s] = -1.0
    while sum(cnt) > nel:
        cand = [k for k in range(nseg) if cnt[k] > 1]
        if not cand:
            break
        s = max(cand, key=lambda k: (cnt[k], -k))
        cnt[s] -= 1
    knots = [lo] * (p + 1)
    for s in range(nseg):
        a, b = brk[s], brk[s + 1]
        knots += [a + (b - a) * i / cnt[s] for i in range(1, cnt[s])]
        if s + 1 < nseg:
            knots += [b] * p
    return np.array(knots + [hi] * (p + 1), dtype=np.float64)


class Space:
    """Tensor B-spline space on the GPU library side (tdz_space handle)."""

    def __init__(self, knots: Sequence[np.ndarray], degree, nquad: int):
        lib = _lib.load()
        self.dim = len(knots)
        deg = [degree] * self.dim if np.isscalar(degree) else list(degree)
        self.knots = [np.ascontiguousarray(k, dtype=np.float64) for k in knots]
        self.degree = deg
        self.nquad = nquad
        arr_t = C.POINTER(C.c_double) * self.dim
        kp = arr_t(*[_lib.dptr(k) for k in self.knots])
        h = C.c_void_p()
        _lib.check(lib.tdz_space_create(self.dim, (C.c_int * self.dim)(*deg),
                                        (C.c_int * self.dim)(*[len(k) for k in self.knots]), kp, nquad,
                                        C.byref(h)))
        self.handle = h
        self.n, self.nel = [], []
        for d in range(self.dim):
            n, ne, p = C.c_int(), C.c_int(), C.c_int()
            _lib.check(lib.tdz_space_axis(h, d, C.byref(n), C.byref(ne), C.byref(p)))
            self.n.append(n.value)
            self.nel.append(ne.value)

    @property
    def ndof(self) -> int:
        return int(np.prod(self.n))

    @property
    def shape(self):
        return tuple(reversed(self.n))

    def quadrature(self, axis: int):
        m = self.nel[axis] * self.nquad
        x = np.zeros(m)
        w = np.zeros(m)
        _lib.check(_lib.load().tdz_space_quadrature(self.handle, axis, _lib.dptr(x), _lib.dptr(w)))
        return x, w

    def project(self, axis: int, f) -> np.ndarray:
        """L2 load vector sum_q w_q B_i(x_q) f(x_q) of one axis (complex)."""
        x, _ = self.quadrature(axis)
        fq = np.ascontiguousarray(np.asarray(f(x), dtype=np.complex128).view(np.float64))
        out = np.zeros(2 * self.n[axis])
        _lib.check(_lib.load().tdz_space_project(self.handle, axis, _lib.dptr(fq), _lib.dptr(out)))
        return out.view(np.complex128)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().tdz_space_destroy(h)
            except Exception:
                pass
            self.handle = None
