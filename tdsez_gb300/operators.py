"""Host side of the matrix-free operators (tdz_op handle).

``Physics`` describes the carrier the way TDSE-Z's input does (potential,
mass, CAP, polarisation, boundary); it is evaluated at the 1D quadrature
points of the space and handed to ``tdz_operator_create``. ``Operator``
mirrors ``TDSEZTensorOps::Apply`` (``src/tensorops.cpp:155-188``) and the
stage matrices of ``src/propagator.cpp:374-551`` on torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

from . import _lib
from .space import Space

MA_C = 2.62206


def cap_width(kmin: float) -> float:
    """Manolopoulos layer width c / (2 delta kmin), delta = 0.2
    (``src/assembly/assembly.cpp:1892-1895``)."""
    return MA_C / (2.0 * 0.2 * kmin)


def manolopoulos(u: float, width: float, kmin: float) -> float:
    """Manolopoulos CAP at layer coordinate u (``assembly.cpp:170-208``)."""
    c = MA_C
    a = 1.0 - 16.0 / c ** 3
    b = (1.0 - 17.0 / c ** 3) / (c * c)
    emin = 0.5 * kmin * kmin
    rcap = width - c / (2.0 * 0.2 * kmin)
    au = abs(u)
    if au <= rcap:
        return 0.0
    r = c * ((au - rcap) / (width - rcap))
    if au >= width:
        r = c * (1.0 - np.finfo(np.float64).eps)
    return emin * (a * r - b * r ** 3 + 4.0 / (c - r) ** 2 - 4.0 / (c + r) ** 2)


def cap_profile(x: float, lo: float, hi: float, kmin: float) -> float:
    """One-axis CAP W_d(x): layer of width w at both walls (``cap.cpp:31-36``)."""
    w = cap_width(kmin)
    s = min(x - lo, hi - x)
    if not (s < w):
        return 0.0
    return manolopoulos(min(w - s, w * (1.0 - 1e-10)), w, kmin)


@dataclass
class Physics:
    """Separable carrier: V = sum_d V_d(x_d), 1/m constant or a function of
    one axis, Manolopoulos CAP on every axis (kmin), field on ``coupled``."""
    charge: float = -1.0
    mass: float = 1.0
    mass_axis: Optional[int] = None
    inv_mass_fn: Optional[Callable[[float], float]] = None
    potential: Sequence[Optional[Callable[[float], float]]] = ()
    cap_kmin: Optional[float] = None
    bounds: Sequence[tuple] = ()
    coupled: Sequence[int] = (0,)
    dirichlet: bool = False
    # non-separable soft-core centres (Z, cx, cy, cz, a): V(r) += -Z / sqrt(|r - c|^2 + a)
    softcore: Sequence[tuple] = ()

    @property
    def sign(self) -> float:
        return -self.charge


class Operator:
    """M, H (+CAP), D_a and the stage operator A = alpha M + g (H + sum c_a D_a)."""

    def __init__(self, space: Space, phys: Physics):
        lib = _lib.load()
        self.space = space
        self.phys = phys
        st = _lib.tdz_physics()
        st.charge = phys.charge
        st.inv_mass = 1.0 / phys.mass
        st.mass_axis = -1 if phys.mass_axis is None else phys.mass_axis
        self._keep = []
        vec = np.vectorize
        if phys.mass_axis is not None:
            xq, _ = space.quadrature(phys.mass_axis)
            arr = np.ascontiguousarray(vec(phys.inv_mass_fn)(xq), dtype=np.float64)
            self._keep.append(arr)
            st.inv_mass_q = _lib.dptr(arr)
        for d in range(space.dim):
            f = phys.potential[d] if d < len(phys.potential) else None
            if f is not None:
                xq, _ = space.quadrature(d)
                arr = np.ascontiguousarray(vec(f)(xq), dtype=np.float64)
                self._keep.append(arr)
                st.pot_q[d] = _lib.dptr(arr)
            if phys.cap_kmin is not None:
                xq, _ = space.quadrature(d)
                lo, hi = phys.bounds[d]
                arr = np.ascontiguousarray(vec(lambda x: cap_profile(x, lo, hi, phys.cap_kmin))(xq),
                                           dtype=np.float64)
                self._keep.append(arr)
                st.cap_q[d] = _lib.dptr(arr)
        if phys.cap_kmin is not None and phys.mass_axis is not None and space.dim > 1:
            raise ValueError("separable CAP with a position-dependent mass needs 1D")
        st.cap_inv_mass = 1.0 / phys.mass
        for a in phys.coupled:
            if a < space.dim:
                st.coupled[a] = 1
        st.dirichlet = 1 if phys.dirichlet else 0
        if phys.softcore:
            arr = np.ascontiguousarray(np.array([list(c) + [0.0] * (5 - len(c)) if len(c) < 5 else list(c)
                                                 for c in phys.softcore], dtype=np.float64).reshape(-1))
            self._keep.append(arr)
            st.nsoft = len(phys.softcore)
            st.soft = _lib.dptr(arr)
        self.coupled = [a for a in range(space.dim) if st.coupled[a]]
        h = C.c_void_p()
        _lib.check(lib.tdz_operator_create(space.handle, C.byref(st), C.byref(h)))
        self.handle = h

    def set_stage(self, alpha: complex, g: complex, c: Sequence[complex] = ()):
        c = list(c)
        arr = (C.c_double * (2 * max(1, len(c))))()
        for k, v in enumerate(c):
            arr[2 * k] = complex(v).real
            arr[2 * k + 1] = complex(v).imag
        _lib.check(_lib.load().tdz_operator_set_stage(self.handle, complex(alpha).real, complex(alpha).imag,
                                                      complex(g).real, complex(g).imag, len(c), arr))

    def apply(self, which: int, x, y, stream=None, df: bool = False, f32: bool = False):
        """y = op x on torch complex64 / complex128 CUDA tensors. On
        complex128: ``df`` computes in double-float arithmetic (TDZ_FP64_DF),
        ``f32`` in FP32 arithmetic (TDZ_FP64_F32, 3D without soft-core
        centres)."""
        import torch
        if x.dtype != y.dtype or x.dtype not in (torch.complex64, torch.complex128):
            raise TypeError("x and y must both be complex64 or complex128")
        if not (x.is_cuda and y.is_cuda and x.is_contiguous() and y.is_contiguous()):
            raise TypeError("x and y must be contiguous CUDA tensors")
        if x.numel() != self.space.ndof or y.numel() != self.space.ndof:
            raise ValueError("vector length does not match the space")
        prec = _lib.TDZ_FP64 if x.dtype == torch.complex128 else _lib.TDZ_FP32
        if df and prec == _lib.TDZ_FP64:
            prec = _lib.TDZ_FP64_DF
        elif f32 and prec == _lib.TDZ_FP64:
            prec = _lib.TDZ_FP64_F32
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _lib.check(_lib.load().tdz_operator_apply(self.handle, which, prec, C.c_void_p(x.data_ptr()),
                                                  C.c_void_p(y.data_ptr()), C.c_void_p(s)))
        return y

    def observables(self, psi, stream=None):
        """(<psi|M|psi>, <psi|H|psi>, [<psi|D_a|psi>]) of a complex128 CUDA
        state: the monitor expectation values of src/manager.cpp:584-672."""
        import torch
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        out = (C.c_double * (4 + 2 * self.space.dim))()
        _lib.check(_lib.load().tdz_observables(self.handle, C.c_void_p(psi.data_ptr()), out, C.c_void_p(s)))
        return out[0], complex(out[2], out[3]), [complex(out[4 + 2 * a], out[5 + 2 * a]) for a in range(self.space.dim)]

    def mass_solve(self, x, stream=None):
        """x <- M^-1 x in place (complex64 / complex128 CUDA tensor)."""
        import torch
        prec = _lib.TDZ_FP64 if x.dtype == torch.complex128 else _lib.TDZ_FP32
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _lib.check(_lib.load().tdz_operator_mass_solve(self.handle, prec, C.c_void_p(x.data_ptr()), C.c_void_p(s)))
        return x

    def separable_state(self, fns, device="cuda"):
        """M-projection of prod_d f_d(x_d) onto the space (complex128 tensor),
        normalised to psi^H M psi = 1."""
        import torch
        vecs = [torch.tensor(self.space.project(d, fns[d]), device=device) for d in range(self.space.dim)]
        psi = vecs[-1]
        for v in reversed(vecs[:-1]):
            psi = torch.outer(psi, v).reshape(-1)
        psi = psi.contiguous()
        self.mass_solve(psi)
        from . import _lib as L
        m = torch.empty_like(psi)
        self.apply(L.TDZ_MASS, psi, m)
        psi /= torch.sqrt(torch.vdot(psi, m).real)
        return psi

    @property
    def launches(self) -> int:
        return int(_lib.load().tdz_operator_launches(self.handle))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().tdz_operator_destroy(h)
            except Exception:
                pass
            self.handle = None
