"""Oracle (test infrastructure only): timed CPU Crank-Nicolson steps with the
reference's CPU method restated — assembled FP64 matrices, GMRES(30) with
an incomplete LU of the CN matrix (SuperLU ILUTP, fill factor 2, drop
1e-4: the ILU(0) of the reference is not available in scipy),
preconditioner built once and reused (``src/propagator.cpp:125-243``), rtol 1e-10.

Used only as the CPU baseline leg of bench.py: a reduced grid of the same
workload family, so that a bounded sample runs in seconds on the host.
"""
from __future__ import annotations

import math
import time

import numpy as np
import scipy.sparse.linalg as sla

from .bspline import Axis, Space
from .operators import Physics, band_sparse, kron_operators


def cn_steps(workload, seconds: float = 15.0, min_steps: int = 2, rtol: float = 1e-10):
    """CN steps/s of the oracle on ``workload`` (an object with knots, p, nq,
    phys (potential / inv_mass_fn / mass_axis / charge), field, dt, packet)."""
    w = workload
    t_setup = time.time()
    axes = [Axis(k, w.p, w.nq) for k in w.knots]
    S = Space(axes)
    dim = S.dim
    pot = w.phys.potential
    ma = w.phys.mass_axis

    seps = [pot[d] if d < len(pot) else None for d in range(dim)]

    def V(x, y, z):
        r = (x, y, z)
        return sum(seps[d](r[d]) for d in range(dim) if seps[d] is not None)

    if ma is None:
        ph = Physics(dim=dim, charge=w.phys.charge, potential=V, mass_const=w.phys.mass, pot_separable=seps,
                     coupled=w.phys.coupled)
    else:
        f = w.phys.inv_mass_fn
        ph = Physics(dim=dim, charge=w.phys.charge, potential=V, inv_mass=lambda x, y, z: f((x, y, z)[ma]),
                     mass_const=None, mass_axis=ma, pot_separable=seps, coupled=w.phys.coupled)
    Mr, Hr, Dr = kron_operators(S, ph)
    M = Mr.astype(np.complex128).tocsc()
    H = Hr.astype(np.complex128).tocsc()
    T = [D.astype(np.complex128).tocsc() for D in Dr]
    # initial state: M-projection of the separable packet (M^-1 factorises by axis)
    vecs = []
    for d in range(dim):
        ax = axes[d]
        b = ax.basis_matrix(0).T @ (ax.wq.reshape(-1) * w.packet[d](ax.xq.reshape(-1)))
        Md = band_sparse(ax.band(), ax.p).tocsc()
        vecs.append(sla.spsolve(Md, b.astype(np.complex128)))
    psi = vecs[-1]
    for v in reversed(vecs[:-1]):
        psi = np.kron(psi, v)
    psi /= math.sqrt(np.vdot(psi, M @ psi).real)
    dt = w.dt
    s = -w.phys.charge
    t = 0.0
    # preconditioner from the first step's matrix, reused
    c0 = [s * e for e in w.field(0.5 * dt)]
    A0 = (M + 0.5j * dt * (H + sum(ci * Ti for ci, Ti in zip(c0, T)))).tocsc()
    ilu = sla.spilu(A0, drop_tol=1e-4, fill_factor=2.0)
    P = sla.LinearOperator(A0.shape, ilu.solve, dtype=np.complex128)
    steps, its = 0, 0
    t0 = time.time()
    setup = t0 - t_setup
    while steps < min_steps or time.time() - t0 < seconds:
        c = [s * e for e in w.field(t + 0.5 * dt)]
        Am = (M + 0.5j * dt * (H + sum(ci * Ti for ci, Ti in zip(c, T)))).tocsc()
        rhs = M @ psi
        cnt = [0]

        def cb(_):
            cnt[0] += 1
        X, info = sla.gmres(Am, rhs, x0=psi, rtol=rtol, atol=0.0, restart=30, maxiter=200, M=P,
                            callback=cb, callback_type="pr_norm")
        if info != 0:
            raise RuntimeError("oracle CN solve did not converge")
        psi = 2 * X - psi
        its += cnt[0]
        t += dt
        steps += 1
    el = time.time() - t0
    return {"steps": steps, "seconds": el, "steps_per_s": steps / el, "ndof": S.ndof,
            "elements": "x".join(str(a.nel) for a in axes), "its_per_step": its / steps, "setup_s": setup}
