"""Host side of the GPU stage solves and time steppers.

``Solver`` mirrors the stage KSP of ``TDSEZConfigureStageKSP``
(``src/propagator.cpp:315-370``); ``Propagator`` mirrors
``TDSEZPropagator::Evolve`` (Crank-Nicolson) and ``EvolveRational``
(Pade(2,2), Magnus-4) of ``src/propagator.cpp:78-769``: step times
t_k = k dt, the last step shortened to end exactly at FinalTime, field
coefficients c_a = s E_a(t) of the coupled axes, and a monitor callback
after every step (``TDSEZMonitorStep``).
"""
from __future__ import annotations

import ctypes as C
import math
import warnings
from typing import Callable, Optional, Sequence

from . import _lib
from .operators import Operator

KINDS = {"cn": _lib.TDZ_CN, "pade22": _lib.TDZ_PADE22, "magnus4": _lib.TDZ_MAGNUS4}
PCS = {"none": _lib.TDZ_PC_NONE, "mass": _lib.TDZ_PC_MASS, "mg": _lib.TDZ_PC_MG, "fdm": _lib.TDZ_PC_FDM,
       "band": _lib.TDZ_PC_BAND}
S3 = math.sqrt(3.0)
MAGNUS_C = (0.5 - S3 / 6.0, 0.5 + S3 / 6.0)


def solver_opts(pc: str = "mg", precision: str = "fp32", rtol: float = 1e-12, restart: int = 0,
                maxit: int = 1000, mg_levels: int = 0, mg_smooth: int = 0, mg_coarse_its: int = 12,
                outer: str = "fp64", mg_learned: bool = False, relaxed: bool = False, pc_refresh_its: int = 0,
                mg_coarse: str = "chebyshev"):
    """Solver options. ``precision`` is the preconditioner's arithmetic
    (fp32 = mixed precision); ``outer`` the arithmetic of the FP64 Krylov
    method's operator applies: "fp64" (native) or "df" (double-float on the
    FP32 pipes, about 48 significant bits). ``pc_refresh_its`` > 0 also
    rebuilds a propagator's preconditioner whenever a stage solve takes more
    iterations (-tdsez_pc_refresh_its). ``mg_coarse``: "chebyshev" (the
    polynomial of degree mg_coarse_its) or "fdm" (the exact FDM inverse of
    the coarsest operator where the stage is separable)."""
    o = _lib.tdz_solver_opts()
    o.restart = restart
    o.maxit = maxit
    o.rtol = rtol
    o.pc = PCS[pc]
    o.pc_precision = _lib.TDZ_FP32 if precision == "fp32" else _lib.TDZ_FP64
    o.mg_levels = mg_levels
    o.mg_smooth = mg_smooth
    o.mg_coarse_its = mg_coarse_its
    o.outer_precision = {"fp64": _lib.TDZ_FP64, "df": _lib.TDZ_FP64_DF}[outer]
    o.mg_learned = 1 if mg_learned else 0
    o.relaxed = 1 if relaxed else 0
    o.pc_refresh_its = max(0, int(pc_refresh_its))
    o.mg_coarse = {"chebyshev": 0, "fdm": 1}[mg_coarse]
    return o


def _stream(stream):
    import torch
    return torch.cuda.current_stream().cuda_stream if stream is None else stream


class Solver:
    """FGMRES + preconditioner on the current stage of ``op``."""

    def __init__(self, op: Operator, stream=None, **kw):
        self.op = op
        self.opts = solver_opts(**kw)
        h = C.c_void_p()
        _lib.check(_lib.load().tdz_solver_create(op.handle, C.byref(self.opts), C.c_void_p(_stream(stream)),
                                                 C.byref(h)))
        self.handle = h

    def solve(self, b, x, stream=None):
        its, reason, rn = C.c_int(), C.c_int(), C.c_double()
        _lib.check(_lib.load().tdz_solver_solve(self.handle, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
                                                C.c_void_p(_stream(stream)), C.byref(its), C.byref(reason),
                                                C.byref(rn)))
        return its.value, reason.value, rn.value

    def train_coarse(self, pairs: int = 2000, epochs: int = 10, lr: float = 1e-3, seed: int = 20261203,
                     stream=None) -> float:
        """Train the learned coarse correction (solver created with
        mg_learned=True) on pairs the solver generates; returns the last
        epoch's mean relative loss."""
        loss = C.c_float()
        _lib.check(_lib.load().tdz_solver_train_coarse(self.handle, pairs, epochs, lr, seed, C.byref(loss),
                                                       C.c_void_p(_stream(stream))))
        return loss.value

    def coarse_gain(self, trials: int = 20, seed: int = 7, stream=None):
        """(plain, learned) relative error of the coarsest solve against a
        10x longer solve on fresh right-hand sides."""
        a, b = C.c_double(), C.c_double()
        _lib.check(_lib.load().tdz_solver_coarse_gain(self.handle, trials, seed, C.byref(a), C.byref(b),
                                                      C.c_void_p(_stream(stream))))
        return a.value, b.value

    def precondition(self, r, z, stream=None):
        """z = P^-1 r (complex128 CUDA tensors): one preconditioner application."""
        _lib.check(_lib.load().tdz_solver_precondition(self.handle, C.c_void_p(r.data_ptr()), C.c_void_p(z.data_ptr()),
                                                       C.c_void_p(_stream(stream))))
        return z

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().tdz_solver_destroy(h)
            except Exception:
                pass
            self.handle = None


class Propagator:
    """Crank-Nicolson / Pade(2,2) / Magnus-4 on the GPU.

    ``field(t)`` returns the physical field E_a(t) of the coupled axes; the
    coefficients handed to the library are s E_a(t), s = -Charge."""

    def __init__(self, op: Operator, kind: str = "cn", field: Optional[Callable[[float], Sequence[float]]] = None,
                 guess_order: int = 3, stream=None, **kw):
        """guess_order: 0..5 extrapolates the stage solutions of the previous
        steps (-pade_guess_order); -1 starts each stage solve from the
        preconditioner's answer x0 = P^-1 b (one FGMRES iteration per solve
        with the exact FDM inverse)."""
        self.op = op
        self.kind = kind
        self.field = field or (lambda t: [0.0] * len(op.coupled))
        self.sign = op.phys.sign
        self.opts = solver_opts(**kw)
        h = C.c_void_p()
        _lib.check(_lib.load().tdz_prop_create(op.handle, KINDS[kind], C.byref(self.opts), guess_order,
                                               C.c_void_p(_stream(stream)), C.byref(h)))
        self.handle = h

    def coeffs(self, t: float):
        return [self.sign * e for e in self.field(t)]

    def step(self, psi, t: float, h: float, stream=None):
        """One step from t to t + h on the complex128 CUDA tensor psi (in place)."""
        nc = len(self.op.coupled)
        arr = C.c_double * max(1, nc)
        if self.kind == "magnus4":
            c1 = arr(*self.coeffs(t + MAGNUS_C[0] * h))
            c2 = arr(*self.coeffs(t + MAGNUS_C[1] * h))
        else:
            c1 = arr(*self.coeffs(t + 0.5 * h))
            c2 = None
        _lib.check(_lib.load().tdz_prop_step(self.handle, C.c_void_p(psi.data_ptr()), h, c1, c2,
                                             C.c_void_p(_stream(stream))))
        return psi

    def strong_field_ratio(self, dt: float, final_time: float) -> float:
        """tau max_t sum_a |E_a(t)| L_a over the run (the strong-field check
        of TDSEZSetupMultigrid, src/multigrid.cpp:213-237)."""
        coupled = list(self.op.coupled)

        def fn(axis, t, ctx):
            if axis not in coupled:
                return 0.0
            return float(self.field(t)[coupled.index(axis)])
        cb = _lib.FIELD_FN(fn)
        out = C.c_double()
        _lib.check(_lib.load().tdz_strong_field_ratio(self.op.space.handle, KINDS[self.kind], dt, final_time, cb,
                                                      None, C.byref(out)))
        return out.value

    def evolve(self, psi, dt: float, final_time: float, monitor=None, stream=None):
        """Steps t_k = k dt, the last one shortened to end at final_time
        (``src/propagator.cpp:734-741``); ``monitor(step, t, psi)`` after
        every step and at t = 0. With the multigrid preconditioner a field
        that dominates the stage operator (tau max|E.r| > 1.5) is warned
        about first, as the reference does."""
        if self.opts.pc == PCS["mg"] and not getattr(self, "_field_checked", False):
            self._field_checked = True
            r = self.strong_field_ratio(dt, final_time)
            if r > 1.5:
                warnings.warn("tau*max|E.r| = %.2g > 1.5: the field term dominates the propagator operator and "
                              "multigrid may not converge; use the FDM or mass preconditioner or a smaller "
                              "time step" % r, RuntimeWarning, stacklevel=2)
        n = int(math.ceil(final_time / dt - 1e-9))
        if monitor:
            monitor(0, 0.0, psi)
        for step in range(n):
            t1 = final_time if step + 1 == n else (step + 1) * dt
            h = t1 - step * dt
            if abs(h - dt) <= 1e-12 * dt:
                h = dt
            self.step(psi, step * dt, h, stream)
            if monitor:
                monitor(step + 1, t1, psi)
        return psi

    def stats(self):
        s, i, a, cy, li = C.c_longlong(), C.c_longlong(), C.c_longlong(), C.c_longlong(), C.c_int()
        rr = C.c_double()
        _lib.check(_lib.load().tdz_prop_stats(self.handle, C.byref(s), C.byref(i), C.byref(a), C.byref(cy),
                                              C.byref(li), C.byref(rr)))
        return {"solves": s.value, "its": i.value, "applies": a.value, "cycles": cy.value,
                "last_its": li.value, "last_rres": rr.value}

    def record_coarse(self, capacity: int):
        """Record the coarsest right-hand sides of the next ``capacity``
        V-cycles of each stage solver (pc="mg", mg_learned=True); 0 stops."""
        _lib.check(_lib.load().tdz_prop_record_coarse(self.handle, capacity))

    def train_coarse(self, epochs: int = 30, lr: float = 1e-3, seed: int = 20261203, stream=None):
        """Train the learned coarse correction on the recorded right-hand
        sides; returns (last-epoch loss, pairs)."""
        loss, pairs = C.c_float(), C.c_int()
        _lib.check(_lib.load().tdz_prop_train_coarse(self.handle, epochs, lr, seed, C.byref(loss), C.byref(pairs),
                                                     C.c_void_p(_stream(stream))))
        return loss.value, pairs.value

    def refreshes(self) -> int:
        """Preconditioner rebuilds the refresh rule asked for so far."""
        n = C.c_longlong()
        _lib.check(_lib.load().tdz_prop_refreshes(self.handle, C.byref(n)))
        return n.value

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().tdz_prop_destroy(h)
            except Exception:
                pass
            self.handle = None


class BatchPropagator:
    """Many independent propagations advanced together (intensity / phase
    scans): each run has its own Propagator, state and CUDA stream; one call
    per step (``tdz_prop_step_batch``) steps them concurrently from a pool of
    host threads, so the GPU overlaps the runs' small kernels and host
    synchronisations. Runs may differ in grid, degree, physics and field."""

    def __init__(self, props: Sequence[Propagator], threads: int = 16):
        import torch
        self.props = list(props)
        if len({id(P.op) for P in self.props}) != len(self.props):
            raise ValueError("each run needs its own Operator (the stage coefficients live there)")
        self.threads = threads
        self.streams = [torch.cuda.Stream() for _ in self.props]

    def step(self, psis, t: float, h: float):
        """One step from t to t + h of every run (psis[i]: complex128 CUDA tensors, in place)."""
        import torch
        n = len(self.props)
        for s in self.streams:   # the states were written on the current stream
            s.wait_stream(torch.cuda.current_stream())
        c1s, c2s, keep = [], [], []
        for P in self.props:
            nc = len(P.op.coupled)
            arr = C.c_double * max(1, nc)
            if P.kind == "magnus4":
                a = arr(*P.coeffs(t + MAGNUS_C[0] * h))
                b = arr(*P.coeffs(t + MAGNUS_C[1] * h))
            else:
                a, b = arr(*P.coeffs(t + 0.5 * h)), arr(*([0.0] * max(1, nc)))
            keep += [a, b]
            c1s.append(C.cast(a, C.POINTER(C.c_double)))
            c2s.append(C.cast(b, C.POINTER(C.c_double)))
        VPA = C.c_void_p * n
        DPA = C.POINTER(C.c_double) * n
        _lib.check(_lib.load().tdz_prop_step_batch(
            n, VPA(*[P.handle.value for P in self.props]), VPA(*[p.data_ptr() for p in psis]), h,
            DPA(*c1s), DPA(*c2s), VPA(*[s.cuda_stream for s in self.streams]), self.threads))
        for s in self.streams:
            torch.cuda.current_stream().wait_stream(s)
        return psis
