"""Oracle (test infrastructure only): tensor B-spline spaces on the CPU in FP64.

This module restates, in numpy, the discretisation that TDSE-Z builds through
PetIGA for its propagation path. It is used only by ``tests/``, by the
smoke check and by the CPU baseline leg of ``bench.py``; the product path
never imports it.

Restated reference pieces:

* open uniform knots, ``IGAAxisInitUniform(axis, nel, lo, hi, C = p-1)``
  (``src/core.cpp:1826-1952``): p+1 copies of each end, simple interior knots;
* ``TDSEZExpSymKnots`` (``src/core_knots.cpp:77-120``): symmetric
  exponential grading towards the origin;
* ``TDSEZInterfaceKnots`` (``src/core_knots.cpp:318-385``): elements
  distributed over material layers by largest remainder, multiplicity p at
  every interface;
* the Gauss-Legendre rule of ``src/tsurff.cpp:24-44`` (Newton on P_n);
* the Cox-de Boor recursion of ``src/tsurff.cpp:47-66`` (Piegl-Tiller A2.2),
  extended to first derivatives (Piegl-Tiller A2.3);
* the 1D band matrices of ``src/tensorops.cpp:40-57`` (entry (i, j) at
  ``i*(2p+1) + j-i+p``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


# --------------------------------------------------------------------------
# knot vectors
# --------------------------------------------------------------------------

def uniform_knots(nel: int, lo: float, hi: float, p: int) -> np.ndarray:
    """Open uniform knots with simple interior knots (C^{p-1} basis)."""
    inner = [lo + (hi - lo) * i / nel for i in range(1, nel)]
    return np.array([lo] * (p + 1) + inner + [hi] * (p + 1), dtype=np.float64)


def symexp_knots(lo: float, hi: float, ninterior: int, alpha: float, p: int) -> np.ndarray:
    """Exponentially graded interior knots, symmetric about 0
    (``src/core_knots.cpp:77-120``): t uniform in (-1, 1), s = |t|,
    mapped = (e^{alpha s} - 1) / (e^alpha - 1), knot = mapped * (hi or lo)."""
    k = [lo] * (p + 1)
    for i in range(ninterior):
        t = 2.0 * (i + 1.0) / (ninterior + 1) - 1.0
        s = abs(t)
        mapped = (math.exp(alpha * s) - 1.0) / (math.exp(alpha) - 1.0)
        k.append(mapped * hi if t >= 0.0 else mapped * lo)
    k += [hi] * (p + 1)
    return np.array(k, dtype=np.float64)


def interface_knots(lo: float, hi: float, ninterior: int, p: int, breakpoints) -> np.ndarray:
    """Layer-aligned knots (``src/core_knots.cpp:318-385``): Nelements =
    ninterior + 1 elements distributed over the layers in proportion to their
    width (largest remainder, at least one per layer), uniform inside each
    layer, every interior breakpoint repeated p times (C0 there)."""
    nelements = ninterior + 1
    tol = 1e-9 * (hi - lo)
    brk = [lo]
    for x in sorted(breakpoints):
        if lo + tol < x < hi - tol and x > brk[-1] + tol:
            brk.append(x)
    brk.append(hi)
    nseg = len(brk) - 1
    if nelements < nseg:
        raise ValueError("fewer elements than material segments")
    nel = [1] * nseg
    rem = [0.0] * nseg
    assigned = 0
    for s in range(nseg):
        share = nelements * (brk[s + 1] - brk[s]) / (hi - lo)
        nel[s] = max(1, int(math.floor(share)))
        rem[s] = share - math.floor(share)
        assigned += nel[s]
    while assigned < nelements:
        s = int(np.argmax(rem))
        nel[s] += 1
        rem[s] = -1.0
        assigned += 1
    while assigned > nelements:
        cand = [k for k in range(nseg) if nel[k] > 1]
        if not cand:
            break
        s = max(cand, key=lambda k: (nel[k], -k))
        nel[s] -= 1
        assigned -= 1
    knots = [lo] * (p + 1)
    for s in range(nseg):
        a, b = brk[s], brk[s + 1]
        for i in range(1, nel[s]):
            knots.append(a + (b - a) * i / nel[s])
        if s + 1 < nseg:
            knots += [b] * p
    knots += [hi] * (p + 1)
    return np.array(knots, dtype=np.float64)


# --------------------------------------------------------------------------
# quadrature and basis
# --------------------------------------------------------------------------

def gauss_legendre(n: int):
    """Nodes and weights on [-1, 1] by Newton iteration on the Legendre
    recurrence (``src/tsurff.cpp:24-44``)."""
    x = np.zeros(n)
    w = np.zeros(n)
    for j in range(n):
        z = math.cos(math.pi * (j + 0.75) / (n + 0.5))
        for _ in range(100):
            p, p0 = 1.0, 0.0
            for k in range(1, n + 1):
                p, p0 = ((2 * k - 1) * z * p - (k - 1) * p0) / k, p
            der = n * (z * p - p0) / (z * z - 1)
            dz = p / der
            z -= dz
            if abs(dz) < 1e-15:
                break
        p, p0 = 1.0, 0.0
        for k in range(1, n + 1):
            p, p0 = ((2 * k - 1) * z * p - (k - 1) * p0) / k, p
        der = n * (z * p - p0) / (z * z - 1)
        x[j] = z
        w[j] = 2.0 / ((1 - z * z) * der * der)
    order = np.argsort(x)
    return x[order], w[order]


def find_span(U: np.ndarray, p: int, n: int, x: float) -> int:
    """Span s in [p, n-1] with U[s] <= x < U[s+1] (last span closed)."""
    if x >= U[n]:
        return n - 1
    lo, hi = p, n
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if x < U[mid]:
            hi = mid
        else:
            lo = mid
    return lo


def ders_basis(U: np.ndarray, p: int, s: int, x: float, nd: int = 1) -> np.ndarray:
    """Values and derivatives (rows 0..nd) of the p+1 B-splines that are
    non-zero on span s at x (Piegl-Tiller A2.3)."""
    ndu = np.zeros((p + 1, p + 1))
    left = np.zeros(p + 1)
    right = np.zeros(p + 1)
    ndu[0, 0] = 1.0
    for j in range(1, p + 1):
        left[j] = x - U[s + 1 - j]
        right[j] = U[s + j] - x
        saved = 0.0
        for r in range(j):
            ndu[j, r] = right[r + 1] + left[j - r]
            temp = ndu[r, j - 1] / ndu[j, r]
            ndu[r, j] = saved + right[r + 1] * temp
            saved = left[j - r] * temp
        ndu[j, j] = saved
    ders = np.zeros((nd + 1, p + 1))
    ders[0, :] = ndu[:, p]
    a = np.zeros((2, p + 1))
    for r in range(p + 1):
        s1, s2 = 0, 1
        a[0, 0] = 1.0
        for k in range(1, nd + 1):
            d = 0.0
            rk, pk = r - k, p - k
            if r >= k:
                a[s2, 0] = a[s1, 0] / ndu[pk + 1, rk]
                d = a[s2, 0] * ndu[rk, pk]
            j1 = 1 if rk >= -1 else -rk
            j2 = k - 1 if r - 1 <= pk else p - r
            for j in range(j1, j2 + 1):
                a[s2, j] = (a[s1, j] - a[s1, j - 1]) / ndu[pk + 1, rk + j]
                d += a[s2, j] * ndu[rk + j, pk]
            if r <= pk:
                a[s2, k] = -a[s1, k - 1] / ndu[pk + 1, r]
                d += a[s2, k] * ndu[r, pk]
            ders[k, r] = d
            s1, s2 = s2, s1
    fac = p
    for k in range(1, nd + 1):
        ders[k, :] *= fac
        fac *= p - k
    return ders


@dataclass
class Axis:
    """One axis of the tensor space: knots, degree, element quadrature and
    basis tables (the data of one PetIGA ``IGABasis``)."""
    knots: np.ndarray
    p: int
    nq: int
    n: int = 0
    spans: np.ndarray = field(default=None)       # knot span index per element
    offset: np.ndarray = field(default=None)      # first basis index per element
    xq: np.ndarray = field(default=None)          # (nel, nq) quadrature points
    wq: np.ndarray = field(default=None)          # (nel, nq) weights * detJac
    N: np.ndarray = field(default=None)           # (nel, nq, p+1) values
    dN: np.ndarray = field(default=None)          # (nel, nq, p+1) first derivatives

    def __post_init__(self):
        U = np.asarray(self.knots, dtype=np.float64)
        self.knots = U
        p = self.p
        self.n = len(U) - p - 1
        spans = [k for k in range(p, self.n) if U[k + 1] > U[k]]
        self.spans = np.array(spans, dtype=np.int64)
        self.offset = self.spans - p
        gx, gw = gauss_legendre(self.nq)
        nel = len(spans)
        self.xq = np.zeros((nel, self.nq))
        self.wq = np.zeros((nel, self.nq))
        self.N = np.zeros((nel, self.nq, p + 1))
        self.dN = np.zeros((nel, self.nq, p + 1))
        for e, s in enumerate(spans):
            a, b = U[s], U[s + 1]
            for q in range(self.nq):
                x = 0.5 * (a + b) + 0.5 * (b - a) * gx[q]
                self.xq[e, q] = x
                self.wq[e, q] = gw[q] * 0.5 * (b - a)
                d = ders_basis(U, p, s, x, 1)
                self.N[e, q] = d[0]
                self.dN[e, q] = d[1]

    @property
    def nel(self) -> int:
        return len(self.spans)

    def basis_matrix(self, deriv: int = 0):
        """Sparse (nel*nq) x n matrix of basis values (or derivatives) at the
        quadrature points, element-major."""
        import scipy.sparse as sp
        T = self.dN if deriv else self.N
        nel, nq, pp = T.shape
        rows = np.repeat(np.arange(nel * nq), pp)
        cols = (self.offset[:, None, None] + np.arange(pp)[None, None, :]).repeat(nq, axis=1).reshape(-1)
        return sp.csr_matrix((T.reshape(-1), (rows, cols)), shape=(nel * nq, self.n))

    def band(self, weight=None, da: int = 0, db: int = 0) -> np.ndarray:
        """1D band (n, 2p+1): A[i, j-i+p] = sum_q w_q f(x_q) B_i^(da) B_j^(db)
        (``src/tensorops.cpp:40-57``). ``weight`` is None, a callable of x or
        an array of values at the quadrature points (nel, nq)."""
        p, bw = self.p, 2 * self.p + 1
        A = np.zeros((self.n, bw))
        if weight is None:
            f = np.ones_like(self.xq)
        elif callable(weight):
            f = np.vectorize(weight)(self.xq)
        else:
            f = np.asarray(weight, dtype=np.float64).reshape(self.xq.shape)
        Ta = self.dN if da else self.N
        Tb = self.dN if db else self.N
        for e in range(self.nel):
            o = self.offset[e]
            E = np.einsum("q,qa,qb->ab", self.wq[e] * f[e], Ta[e], Tb[e])
            for a in range(p + 1):
                for b in range(p + 1):
                    A[o + a, b - a + p] += E[a, b]
        return A

    def greville(self) -> np.ndarray:
        p = self.p
        U = self.knots
        return np.array([U[i + 1:i + p + 1].sum() / max(p, 1) for i in range(self.n)])


def band_to_dense(A: np.ndarray, p: int) -> np.ndarray:
    n = A.shape[0]
    D = np.zeros((n, n), dtype=A.dtype)
    for i in range(n):
        for j in range(max(0, i - p), min(n, i + p + 1)):
            D[i, j] = A[i, j - i + p]
    return D


def dense_to_band(D: np.ndarray, p: int) -> np.ndarray:
    n = D.shape[0]
    A = np.zeros((n, 2 * p + 1), dtype=D.dtype)
    for i in range(n):
        for j in range(max(0, i - p), min(n, i + p + 1)):
            A[i, j - i + p] = D[i, j]
    return A


class Space:
    """Tensor B-spline space, x fastest (natural ordering of
    ``src/tensorops.cpp:133-136``)."""

    def __init__(self, axes):
        self.axes = list(axes)
        self.dim = len(self.axes)

    @property
    def shape(self):
        """Coefficient array shape, slowest axis first: (n_z, n_y, n_x)."""
        return tuple(a.n for a in reversed(self.axes))

    @property
    def ndof(self) -> int:
        return int(np.prod([a.n for a in self.axes]))

    def quad_coords(self):
        """Coordinates of all tensor quadrature points, arrays shaped like the
        quadrature grid (slowest axis first)."""
        xs = [a.xq.reshape(-1) for a in self.axes]
        grids = np.meshgrid(*reversed(xs), indexing="ij")
        return list(reversed(grids))

    def quad_weights(self):
        ws = [a.wq.reshape(-1) for a in self.axes]
        W = ws[-1]
        for w in reversed(ws[:-1]):
            W = np.multiply.outer(W, w)
        return W
