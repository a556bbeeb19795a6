"""Oracle (test infrastructure only): Crank-Nicolson, Pade(2,2) and Magnus-4
steps on the assembled FP64 matrices, solved directly (sparse LU).

* Crank-Nicolson is PETSc ``TSTHETA`` with theta = 1/2 and no endpoint
  (``src/propagator.cpp:94-101``): with the IFunction/IJacobian of
  ``src/monitor.cpp:273-331`` the stage equation is
  (M + i h/2 H_E(t + h/2)) X = M psi_n and psi_{n+1} = 2 X - psi_n.
* Pade(2,2) (``src/propagator.cpp:564-676``): two Cayley stages
  (M + g_k H_E) y = (M + conj(g_k) H_E) x, g_{1,2} = h(-+sqrt3 + 3i)/12, the
  right-hand side formed as 2 M x - A_other x.
* Magnus-4 (``src/propagator.cpp:682-769``): two Pade(2,2) half steps with the
  effective field coefficients 2(a2 c(t+c1 h) + a1 c(t+c2 h)) then
  2(a1 c(t+c1 h) + a2 c(t+c2 h)); c_{1,2} = 1/2 -+ sqrt3/6,
  a_{1,2} = (3 -+ 2 sqrt3)/12.
* Field coefficients c_a(t) = s E_a(t) on the coupled axes
  (``TDSEZManager::TermCoefficients``, ``src/manager.cpp:1020-1027``).
"""
from __future__ import annotations

import math
from typing import Callable, Sequence

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from .operators import Assembled

S3 = math.sqrt(3.0)
PADE_G = (complex(-S3, 3.0) / 12.0, complex(S3, 3.0) / 12.0)
MAGNUS_C = (0.5 - S3 / 6.0, 0.5 + S3 / 6.0)
MAGNUS_A = ((3.0 - 2.0 * S3) / 12.0, (3.0 + 2.0 * S3) / 12.0)


class OraclePropagator:
    """Time stepping on the assembled operators of ``asm``.

    ``field(t)`` returns the physical field components E_a(t) of the coupled
    axes (in ``asm.phys.coupled`` order)."""

    def __init__(self, asm: Assembled, field: Callable[[float], Sequence[float]], kind: str = "cn"):
        self.asm = asm
        self.kind = kind
        self.field = field
        self.M = asm.M.astype(np.complex128).tocsc()
        self.H = asm.H_total().astype(np.complex128).tocsc()
        self.T = [D.astype(np.complex128).tocsc() for D in asm.terms()]
        self.s = asm.phys.sign
        self._lu = {}     # (scale, coefficients) -> LU of M + scale H_E, for repeated stages

    def _solve(self, scale, c, rhs):
        """(M + scale H_E(c))^-1 rhs by a sparse LU, kept while the stage
        repeats (a field that is off, or constant)."""
        key = (complex(scale), tuple(complex(v) for v in c))
        lu = self._lu.get(key)
        if lu is None:
            if len(self._lu) >= 4:
                self._lu.clear()
            lu = sla.splu((self.M + scale * self.H_E(c)).tocsc())
            self._lu[key] = lu
        return lu.solve(rhs)

    def coeffs(self, t: float):
        return [self.s * e for e in self.field(t)]

    def H_E(self, c):
        A = self.H.copy()
        for ci, T in zip(c, self.T):
            if ci != 0:
                A = A + ci * T
        return A

    def cn_step(self, psi, t, h):
        X = self._solve(0.5j * h, self.coeffs(t + 0.5 * h), self.M @ psi)
        return 2.0 * X - psi

    def pade_step(self, psi, h, c):
        HE = self.H_E(c)
        A = [(self.M + (g * h) * HE).tocsc() for g in PADE_G]
        x = psi
        for k in range(2):
            rhs = 2.0 * (self.M @ x) - A[1 - k] @ x
            x = self._solve(PADE_G[k] * h, c, rhs)
        return x

    def step(self, psi, t, h):
        if self.kind == "cn":
            return self.cn_step(psi, t, h)
        if self.kind == "pade22":
            return self.pade_step(psi, h, self.coeffs(t + 0.5 * h))
        if self.kind == "magnus4":
            E1 = self.coeffs(t + MAGNUS_C[0] * h)
            E2 = self.coeffs(t + MAGNUS_C[1] * h)
            a1, a2 = MAGNUS_A
            Ea = [2.0 * (a2 * e1 + a1 * e2) for e1, e2 in zip(E1, E2)]
            Eb = [2.0 * (a1 * e1 + a2 * e2) for e1, e2 in zip(E1, E2)]
            psi = self.pade_step(psi, 0.5 * h, Ea)
            return self.pade_step(psi, 0.5 * h, Eb)
        raise ValueError(self.kind)

    def evolve(self, psi, dt, T, observe=None):
        """Steps t_k = k dt, the last one shortened to end at T
        (``src/propagator.cpp:734-741``)."""
        n = int(math.ceil(T / dt - 1e-9))
        out = []
        if observe:
            out.append(observe(0.0, psi))
        for step in range(n):
            t1 = T if step + 1 == n else (step + 1) * dt
            h = t1 - step * dt
            if abs(h - dt) <= 1e-12 * dt:
                h = dt
            psi = self.step(psi, step * dt, h)
            if observe:
                out.append(observe(t1, psi))
        return psi, out


def ground_state(asm: Assembled, target: float = 0.0, k: int = 1):
    """Lowest eigenpair(s) of H c = E M c near ``target`` by shift-invert,
    M-normalised (the role of ``src/core.cpp:887-931``)."""
    H = asm.H.astype(np.float64) if not np.iscomplexobj(asm.H.data) else asm.H.real
    M = asm.M.astype(np.float64)
    n = H.shape[0]
    if n <= 2500:
        import scipy.linalg as la
        E, V = la.eigh(H.toarray(), M.toarray())
        idx = np.argsort(np.abs(E - target))[:k]
        idx = idx[np.argsort(E[idx])]
        E, V = E[idx], V[:, idx]
    else:
        E, V = sla.eigsh(H.tocsc(), k=k, M=M.tocsc(), sigma=target, which="LM")
        o = np.argsort(E)
        E, V = E[o], V[:, o]
    for j in range(V.shape[1]):
        V[:, j] /= math.sqrt(V[:, j] @ (M @ V[:, j]))
    return E, V.astype(np.complex128)


def expect(A, psi):
    return np.vdot(psi, A @ psi)


class PCRefreshRule:
    """The preconditioner refresh rule of ``TDSEZPCRefresh::Stale``
    (``include/tdsez_propagator.hpp:17-31``): the first solve after a build
    sets the base; a solve with more than 2 base + 5 iterations, or more than
    ``cap`` when cap >= 0 (``-tdsez_pc_refresh_its``), asks for a rebuild."""

    def __init__(self, cap: int = -1):
        self.base, self.rebuilds, self.cap = -1, 0, cap

    def stale(self, its: int) -> bool:
        if self.cap >= 0 and its > self.cap:
            self.base = -1
            self.rebuilds += 1
            return True
        if self.base < 0:
            self.base = its
            return False
        if its <= 2 * self.base + 5:
            return False
        self.base = -1
        self.rebuilds += 1
        return True


def strong_field_ratio(kind: str, dt: float, final_time: float, field, bounds) -> float:
    """tau max_t sum_a |E_a(t)| L_a of ``TDSEZSetupMultigrid``'s strong-field
    check (``src/multigrid.cpp:213-237``): 4 T/dt + 1 equispaced samples of
    [0, T], L_a = max(|lo_a|, |hi_a|), tau = dt/2 (CN), dt/sqrt12 (Pade(2,2)),
    dt/(2 sqrt12) (Magnus-4). ``field(a, t)`` is the physical field."""
    tau = {"cn": 0.5 * dt, "pade22": dt / math.sqrt(12.0), "magnus4": dt / (2.0 * math.sqrt(12.0))}[kind]
    L = [max(abs(lo), abs(hi)) for lo, hi in bounds]
    n = int(math.ceil(4.0 * final_time / dt))
    worst = 0.0
    for i in range(n + 1):
        t = final_time * i / max(n, 1)
        worst = max(worst, sum(abs(field(a, t)) * L[a] for a in range(len(L))))
    return tau * worst
