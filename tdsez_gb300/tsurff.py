"""Host side of the GPU t-SURFF sampler (mirrors TDSEZTSurff::Setup/Sample,
``src/tsurff.cpp:112-469``): the flux is added on every OutputStrideSurff-th
step and at FinalTime."""
from __future__ import annotations

import ctypes as C
from typing import Callable, Sequence

import numpy as np

from . import _lib
from .space import Space


class TSurff:
    def __init__(self, space: Space, radius: float, kgrid: Sequence[tuple], field: Callable[[float], Sequence[float]],
                 dt: float, mass: float = 1.0, v0: float = 0.0, charge: float = -1.0, nquad: int = 0,
                 stride: int = 1):
        """kgrid: per axis (kmin, kmax, nk); field(t) -> E_a(t) for every axis."""
        self.space = space
        self.stride = stride
        o = _lib.tdz_tsurff_opts()
        o.radius = radius
        o.nquad = nquad
        for d in range(space.dim):
            o.kmin[d], o.kmax[d], o.nk[d] = kgrid[d][0], kgrid[d][1], int(kgrid[d][2])
        o.mass, o.v0, o.charge, o.dt = mass, v0, charge, dt
        self.nk = [int(kgrid[d][2]) for d in range(space.dim)]
        self.kgrid = [(float(kgrid[d][0]), float(kgrid[d][1]), int(kgrid[d][2])) for d in range(space.dim)]

        def cb(axis, t, ctx):
            try:
                e = field(t)
                return float(e[axis]) if axis < len(e) else 0.0
            except Exception:
                return 0.0
        self._cb = _lib.FIELD_FN(cb)
        h = C.c_void_p()
        _lib.check(_lib.load().tdz_tsurff_create(space.handle, C.byref(o), self._cb, None, C.byref(h)))
        self.handle = h

    def k_axes(self):
        """Momentum axes of the grid, the values the sampler uses:
        k_i = kmin + i (kmax - kmin) / (nk - 1)."""
        return [np.array([lo if n == 1 else lo + i * (hi - lo) / (n - 1) for i in range(n)])
                for lo, hi, n in self.kgrid]

    def sample(self, t: float, psi, stream=None):
        import torch
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _lib.check(_lib.load().tdz_tsurff_sample(self.handle, t, C.c_void_p(psi.data_ptr()), C.c_void_p(s)))

    def amplitudes(self, stream=None) -> np.ndarray:
        import torch
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        out = np.zeros(2 * int(np.prod(self.nk)))
        _lib.check(_lib.load().tdz_tsurff_amplitudes(self.handle, _lib.dptr(out), C.c_void_p(s)))
        return out.view(np.complex128)

    def interior(self, psi, stream=None) -> np.ndarray:
        """Projection of psi inside |x_d| < R onto the Volkov states at the
        last sample time (``Interior``, ``src/tsurff.cpp:565-639``): add it to
        ``amplitudes()`` for the spectrum of a run that ends early."""
        import torch
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        out = np.zeros(2 * int(np.prod(self.nk)))
        _lib.check(_lib.load().tdz_tsurff_interior(self.handle, C.c_void_p(psi.data_ptr()), _lib.dptr(out),
                                                   C.c_void_p(s)))
        return out.view(np.complex128)

    def end_term(self, op, psi, cap_width: float = 0.0, dp: float = 0.0, eta: float = -1.0, rtol: float = 1e-10,
                 maxit: int = 0, inner=None, stream=None):
        """Flux after the last sample time T of a run that ends after the
        pulse (``EndTerm``, ``src/tsurff.cpp:650-976``): amplitudes to add to
        ``amplitudes()``, and a dict of what it took. ``op`` is the field-free
        Hamiltonian's operator with its absorbing layer, ``psi`` = psi(T)
        (sampled at T first), ``cap_width`` the layer width
        (``operators.cap_width(kmin)``; needed when dp = 0), ``inner`` solver
        options (``propagator.solver_opts``; None: banded LU in 1D, FDM in
        2D/3D)."""
        o = _lib.tdz_tsurff_end_opts()
        o.dp, o.cap_width, o.eta, o.rtol, o.maxit = dp, cap_width, eta, rtol, maxit
        out = np.zeros(2 * int(np.prod(self.nk)))
        st = np.zeros(7)
        inner_p = C.cast(C.byref(inner), C.c_void_p) if inner is not None else None
        import torch
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _lib.check(_lib.load().tdz_tsurff_end_term(self.handle, op.handle, inner_p, C.cast(C.byref(o), C.c_void_p),
                                                   C.c_void_p(psi.data_ptr()), _lib.dptr(out), _lib.dptr(st),
                                                   C.c_void_p(s)))
        stats = {"nodes": int(st[0]), "its": int(st[1]), "max_its": int(st[2]), "dp_max": float(st[3]),
                 "eta": float(st[4]), "seconds": float(st[5]), "damped": int(st[6])}
        return out.view(np.complex128), stats

    def volkov(self):
        out = np.zeros(8)
        _lib.check(_lib.load().tdz_tsurff_volkov(self.handle, _lib.dptr(out)))
        return out

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().tdz_tsurff_destroy(h)
            except Exception:
                pass
            self.handle = None
