"""Bound states on the GPU: the shift-invert eigensolve of
``src/core.cpp:887-1048`` (``tdz_eigen_solve``)."""
from __future__ import annotations

import ctypes as C
from typing import Optional

from . import _lib
from .operators import Operator


def bound_states(op: Operator, nev: int = 1, target: float = 0.0, tol: float = 1e-10, maxit: int = 500,
                 start=None, stream=None, **inner):
    """The ``nev`` eigenpairs of H c = E M c nearest ``target`` in FP64.

    ``start``: a complex128 CUDA vector (its real part is the Lanczos start);
    default: the M-projection of a broad separable Gaussian. ``inner``:
    solver options of the shift-invert solves (``pc``, ``precision``,
    ``rtol``, ... as for ``Solver``); default: the FDM inverse in 3D, the
    multigrid otherwise. Returns (energies, vectors (nev, ndof) complex128,
    backward errors, inner solves)."""
    import numpy as np
    import torch
    from .propagator import solver_opts
    n = op.space.ndof
    vecs = torch.zeros((nev, n), dtype=torch.complex128, device="cuda")
    if start is None:
        fns = []
        for d in range(op.space.dim):
            xq, _ = op.space.quadrature(d)
            lo, hi = float(np.min(xq)), float(np.max(xq))
            c, w = 0.5 * (lo + hi), 0.25 * (hi - lo)
            fns.append(lambda x, c=c, w=w: np.exp(-((x - c) / w) ** 2))
        start = op.separable_state(fns)
    vecs[0].copy_(start)
    E = (C.c_double * nev)()
    B = (C.c_double * nev)()
    ns = C.c_int()
    opts = C.byref(solver_opts(**inner)) if inner else None
    s = torch.cuda.current_stream().cuda_stream if stream is None else stream
    _lib.check(_lib.load().tdz_eigen_solve(op.handle, nev, target, tol, maxit, opts, C.c_void_p(vecs.data_ptr()),
                                           E, B, C.byref(ns), C.c_void_p(s)))
    return list(E), vecs, list(B), ns.value
