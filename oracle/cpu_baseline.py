"""Oracle (test infrastructure only): timed CPU Crank-Nicolson steps with the
reference's CPU method restated, on assembled FP64 matrices
(``src/propagator.cpp:125-243``), rtol 1e-10:

* ``cn_steps``: scipy GMRES(30) with an incomplete LU of the CN matrix
  (SuperLU ILUTP, fill factor 2, drop 1e-4), one core;
* ``cn_steps_threads``: the C restatement in ``cn_bjilu.c``: GMRES(30) with
  PETSc's parallel default preconditioner, block Jacobi with ILU(0) per
  block (one block per thread, as one per MPI rank), OpenMP over the host's
  cores.

Both build the preconditioner once from the first step's matrix and reuse
it. Used only as the CPU baseline leg of bench.py and its tests: a reduced
grid of the same workload family, so that a bounded sample runs in seconds.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import platform
import subprocess
import time
from pathlib import Path

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from .bspline import Axis, Space
from .operators import Physics, band_sparse, kron_operators

HERE = Path(__file__).resolve().parent
CLIB = HERE / "_build" / f"libcnbj_{platform.machine()}.so"   # per host architecture


def build_c(force: bool = False) -> Path:
    """Compile cn_bjilu.c (gcc, OpenMP) into oracle/_build when it is stale."""
    src = HERE / "cn_bjilu.c"
    if CLIB.exists() and not force and CLIB.stat().st_mtime >= src.stat().st_mtime:
        return CLIB
    CLIB.parent.mkdir(exist_ok=True)
    tmp = CLIB.with_suffix(".tmp.so")
    subprocess.run(["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"],
                   check=True, capture_output=True, text=True)
    os.replace(tmp, CLIB)
    return CLIB


def _problem(workload):
    """Assembled M, H, dipoles and the initial state of a workload."""
    w = workload
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
    return S, axes, M, H, T, psi


def cn_steps(workload, seconds: float = 15.0, min_steps: int = 2, rtol: float = 1e-10):
    """CN steps/s of the scipy restatement on ``workload`` (an object with knots,
    p, nq, phys (potential / inv_mass_fn / mass_axis / charge), field, dt, packet)."""
    w = workload
    t_setup = time.time()
    S, axes, M, H, T, psi = _problem(w)
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


def _on_pattern(mats):
    """CSR pattern (sorted) of the union of ``mats`` and each matrix's values on it."""
    mats = [m.tocsr() for m in mats]
    for m in mats:
        m.sum_duplicates()
        m.sort_indices()
    pat = abs(mats[0])
    for m in mats[1:]:
        pat = pat + abs(m)
    pat = pat.tocsr()
    pat.sum_duplicates()
    pat.sort_indices()
    n = pat.shape[0]
    prow = np.repeat(np.arange(n, dtype=np.int64), np.diff(pat.indptr))
    pkey = prow * n + pat.indices.astype(np.int64)
    vals = []
    for m in mats:
        mrow = np.repeat(np.arange(n, dtype=np.int64), np.diff(m.indptr))
        pos = np.searchsorted(pkey, mrow * n + m.indices.astype(np.int64))
        v = np.zeros(pat.nnz, dtype=np.complex128)
        v[pos] = m.data
        vals.append(v)
    return pat.indptr.astype(np.int32), pat.indices.astype(np.int32), vals


def cn_steps_threads(workload, seconds: float = 15.0, min_steps: int = 2, rtol: float = 1e-10,
                     threads: int = 0, blocks: int = 1, steps_max: int = 20000, psi=None,
                     return_state: bool = False):
    """CN steps/s of the C restatement (block Jacobi ILU(0) GMRES, OpenMP) on
    ``workload``; threads = 0 uses every host core, blocks = 0 one block per
    thread (the reference on that many MPI ranks), 1 the ILU(0) of the whole
    matrix (its triangular solves sequential, everything else threaded)."""
    w = workload
    S, axes, M, H, T, psi0 = _problem(w)
    psi = (psi0 if psi is None else np.asarray(psi, dtype=np.complex128)).copy()
    rp, ci, vals = _on_pattern([M, H] + list(T))
    nd = len(T)
    s = -w.phys.charge
    dt = w.dt
    nmax = int(steps_max)
    coef = np.zeros((nmax, max(nd, 1)))   # row k: s E_a((k + 1/2) dt) of the coupled axes
    for k in range(nmax):
        coef[k, :nd] = [s * e for e in w.field((k + 0.5) * dt)]
    lib = C.CDLL(str(build_c()))
    f = lib.cn_bjilu_run
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_int,
                  C.c_int, C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    allv = np.ascontiguousarray(np.concatenate(vals))
    out = np.zeros(5)
    psi = np.ascontiguousarray(psi)
    st = f(S.ndof, rp.ctypes.data, ci.ctypes.data, allv.ctypes.data, nd, np.ascontiguousarray(coef).ctypes.data, dt,
           rtol, int(threads), int(blocks), float(seconds), int(min_steps), nmax, psi.ctypes.data, out.ctypes.data)
    if st != 0:
        raise RuntimeError("C CN solver failed (status %d)" % st)
    steps, el, its, nthr, nb = int(out[0]), float(out[1]), int(out[2]), int(out[3]), int(out[4])
    r = {"steps": steps, "seconds": el, "steps_per_s": steps / el if el > 0 else float("inf"), "ndof": S.ndof,
         "elements": "x".join(str(a.nel) for a in axes), "its_per_step": its / max(steps, 1), "threads": nthr,
         "blocks": nb}
    if return_state:
        r["psi"] = psi
    return r
