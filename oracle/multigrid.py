"""Oracle (test infrastructure only): the geometric B-spline multigrid
hierarchy of ``src/multigrid.cpp``.

* ``coarsen_knots``: drop every other simple interior breakpoint, keep
  repeated (C0) knots (``multigrid.cpp:25-40``);
* ``prolongation``: fine coefficients from coarse ones by inserting the
  missing knots one at a time (Boehm), rows sparse (``multigrid.cpp:52-81``);
* ``greville``: Greville abscissae (``multigrid.cpp:84-93``);
* ``hierarchy``: coarsen every axis while it keeps >= p+1 spans, until
  ``levels`` levels or fewer than 2000 DoFs (``multigrid.cpp:239-263``);
* Galerkin coarse operators P^T A P (``PC_MG_GALERKIN_BOTH``,
  ``multigrid.cpp:277``).
"""
from __future__ import annotations

import bisect

import numpy as np
import scipy.sparse as sp


def coarsen_knots(U):
    bp = []
    for u in U:
        if bp and u == bp[-1][0]:
            bp[-1][1] += 1
        else:
            bp.append([u, 1])
    C = []
    dropped = False
    for i, (u, m) in enumerate(bp):
        interior = 0 < i < len(bp) - 1
        if interior and m == 1 and i % 2 == 1:
            dropped = True
            continue
        C += [u] * m
    return np.array(C), dropped


def spans(U) -> int:
    return int(sum(1 for i in range(len(U) - 1) if U[i + 1] > U[i]))


def prolongation(C, F, p: int) -> np.ndarray:
    """Dense (n_fine x n_coarse) Boehm prolongation."""
    U = list(C)
    nc = len(C) - p - 1
    P = np.eye(nc)
    # multiset difference F \ C
    add = []
    i = j = 0
    Cl, Fl = list(C), list(F)
    while i < len(Fl):
        if j < len(Cl) and Cl[j] == Fl[i]:
            i += 1
            j += 1
        elif j < len(Cl) and Cl[j] < Fl[i]:
            j += 1
        else:
            add.append(Fl[i])
            i += 1
    for xi in add:
        n = len(U) - p - 1
        k = bisect.bisect_right(U, xi) - 1
        k = min(max(k, p), n - 1)
        Q = np.zeros((n + 1, nc))
        Q[: k - p + 1] = P[: k - p + 1]
        Q[k + 1:] = P[k:]
        for r in range(k - p + 1, k + 1):
            a = (xi - U[r]) / (U[r + p] - U[r])
            Q[r] = a * P[r] + (1 - a) * P[r - 1]
        P = Q
        U.insert(bisect.bisect_right(U, xi), xi)
    P[np.abs(P) < 1e-14] = 0.0
    return P


def greville(U, p: int) -> np.ndarray:
    n = len(U) - p - 1
    return np.array([sum(U[i + 1:i + p + 1]) / max(p, 1) for i in range(n)])


def hierarchy(knots_per_axis, p, levels: int = 0, min_dofs: int = 2000):
    """List of per-level knot lists (finest first)."""
    K = [list(knots_per_axis)]
    max_levels = levels if levels > 0 else 20
    while len(K) < max_levels:
        Cl = list(K[-1])
        anyc = False
        dofs = 1
        for d, U in enumerate(K[-1]):
            Cd, dropped = coarsen_knots(U)
            if dropped and spans(Cd) >= p + 1:
                Cl[d] = Cd
                anyc = True
            dofs *= len(Cl[d]) - p - 1
        if not anyc:
            break
        K.append(Cl)
        if levels == 0 and dofs < min_dofs:
            break
    return K


def kron_prolongation(Ps):
    """Tensor prolongation, x first in ``Ps`` (x-fastest ordering)."""
    out = sp.csr_matrix(Ps[-1])
    for P in reversed(Ps[:-1]):
        out = sp.kron(out, sp.csr_matrix(P), format="csr")
    return out
