"""Output files of a propagation in the reference's HDF5 schema, written by
libtdz itself (no HDF5 library is linked; any HDF5 reader opens them):

* ``ObservablesFile`` -- ``td/<name>_observables.h5``, five float64 datasets
  with one row per recorded step (TDSEZManager::WriteHDF5,
  ``src/manager.cpp:51-201``);
* ``ObservablesMonitor`` -- a ``Propagator.evolve`` monitor that computes the
  rows on the GPU and records them;
* ``write_surff`` -- ``td/<name>_surff.h5``, the t-SURFF spectra with their
  file attributes (``src/tsurff.cpp:1018-1057``);
* ``write_h5`` -- any flat file of float64 datasets and attributes.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Callable, Mapping, Optional, Sequence

import numpy as np

from . import _lib

SETS = ("dipoles", "populations", "energies", "currents", "autocorrelation")


def write_h5(path: str, datasets: Mapping[str, np.ndarray], attrs: Optional[Mapping[str, object]] = None) -> None:
    """Write ``datasets`` (name -> array of rank 1..8, stored as float64) in
    the root group of ``path`` and ``attrs`` (name -> number or 1D array,
    float64) on it, through ``tdz_h5_write``."""
    names = list(datasets)
    arrs = [np.ascontiguousarray(np.asarray(datasets[n], dtype=np.float64)) for n in names]
    for n, a in zip(names, arrs):
        if a.ndim < 1:
            raise ValueError(f"dataset {n!r} must have rank >= 1")
    attrs = dict(attrs or {})
    anames = list(attrs)
    avals = [np.ascontiguousarray(np.atleast_1d(np.asarray(attrs[n], dtype=np.float64)).reshape(-1)) for n in anames]
    dims = [d for a in arrs for d in a.shape]
    cn = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
    ranks = (C.c_int * max(1, len(names)))(*[a.ndim for a in arrs])
    cd = (C.c_longlong * max(1, len(dims)))(*dims)
    data = (C.POINTER(C.c_double) * max(1, len(arrs)))(*[_lib.dptr(a) for a in arrs])
    can = (C.c_char_p * max(1, len(anames)))(*[n.encode() for n in anames])
    alen = (C.c_longlong * max(1, len(avals)))(*[a.size for a in avals])
    adata = (C.POINTER(C.c_double) * max(1, len(avals)))(*[_lib.dptr(a) for a in avals])
    _lib.check(_lib.load().tdz_h5_write(str(path).encode(), len(names), cn, ranks, cd, data, len(anames), can, alen,
                                        adata))


class ObservablesFile:
    """The observables file of a run: ``record(t, dipoles=..., ...)`` appends
    one row to each of the five datasets (each given without its time
    column; missing ones are zeros), ``flush()`` writes every row so far,
    ``close()`` flushes and releases the file. Rows are written by themselves
    every ``flush_rows`` rows (the reference's 5000-row buffer)."""

    def __init__(self, path: str, dim: int, n_bound: int = 0, flush_rows: int = 5000):
        h = C.c_void_p()
        _lib.check(_lib.load().tdz_obsfile_open(str(path).encode(), dim, n_bound, flush_rows, C.byref(h)))
        self.handle, self.path, self.dim = h, str(path), dim
        self.columns = {name: _lib.load().tdz_obsfile_columns(h, i) for i, name in enumerate(SETS)}

    def record(self, t: float, **rows) -> None:
        unknown = set(rows) - set(SETS)
        if unknown:
            raise ValueError(f"unknown datasets {sorted(unknown)}")
        keep, ptrs = [], (C.POINTER(C.c_double) * len(SETS))()
        for i, name in enumerate(SETS):
            v = rows.get(name)
            if v is None:
                continue
            a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
            if a.size != self.columns[name] - 1:
                raise ValueError(f"{name}: {a.size} values, expected {self.columns[name] - 1} after the time")
            keep.append(a)
            ptrs[i] = _lib.dptr(a)
        self._need_open()
        _lib.check(_lib.load().tdz_obsfile_record(self.handle, float(t), ptrs))

    @property
    def rows(self):
        """(recorded, written) row counts."""
        self._need_open()
        r, w = C.c_longlong(), C.c_longlong()
        _lib.check(_lib.load().tdz_obsfile_rows(self.handle, C.byref(r), C.byref(w)))
        return r.value, w.value

    def flush(self) -> None:
        self._need_open()
        _lib.check(_lib.load().tdz_obsfile_flush(self.handle))

    def close(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.handle = None
            _lib.check(_lib.load().tdz_obsfile_close(h))

    def _need_open(self):
        if self.handle is None:
            raise ValueError("the observables file is closed")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ObservablesMonitor:
    """Monitor ``(step, t, psi)`` for ``Propagator.evolve`` that records the
    observables of every step (the reference records every step too), all
    computed on the GPU through the C ABI:

    * dipoles: t, E_a(t), D_a = q Re<psi|D_a|psi>; the acceleration A_a is
      not computed (zeros);
    * energies: t, Kin = <psi|K|psi>, Pot = Re<psi|H|psi> - Kin (= <sV>:
      the absorbing potential -iW adds only to the imaginary part),
      Int = s E(t).<psi|r|psi>, Tot = Re<psi|H|psi> + Int, InvMass =
      <psi|1/m|psi>, Norm = <psi|M|psi> (unnormalised expectation values,
      s = -q); K and 1/m are applied by two more operator sets of the same
      space (the kinetic term alone; 1/m as a potential);
    * populations: t, |<phi_n|M|psi>|^2 for the given bound states;
    * autocorrelation: t, <psi(0)|M|psi(t)> with psi(0) the state at the
      first call;
    * currents: time only (zeros).

    ``field(t)`` returns the physical field per axis (E_x, E_y, E_z; shorter
    sequences are padded with zeros); ``op`` is the field-free operator set
    (H with its absorbing layer). Call ``close()`` at the end."""

    def __init__(self, path: str, op, field: Optional[Callable[[float], Sequence[float]]] = None,
                 charge: float = -1.0, bound: Sequence = (), flush_rows: int = 5000):
        self.op, self.field, self.q = op, field, float(charge)
        self.dim = op.space.dim
        self.bound = list(bound)
        self.file = ObservablesFile(path, self.dim, len(self.bound), flush_rows)
        self._mv = None          # M phi_n ..., M psi(0) (device vectors)
        self._out = None
        from .operators import Operator, Physics
        ph = op.phys
        # the kinetic term alone: the same carrier without potential, soft-core centres and CAP
        self.op_kin = Operator(op.space, dataclasses.replace(ph, potential=(), cap_kmin=None, softcore=()))
        self.op_inv = None
        self.inv_mass = 1.0 / ph.mass
        if ph.mass_axis is not None:
            # <1/m> as the expectation value of a potential V = 1/m(x_a) with no kinetic term (s = +1)
            pot = [ph.inv_mass_fn if d == ph.mass_axis else None for d in range(self.dim)]
            self.op_inv = Operator(op.space, Physics(charge=-1.0, mass=math.inf, potential=pot, coupled=(),
                                                     dirichlet=ph.dirichlet))

    def _prepare(self, psi):
        import torch
        mv = []
        for v in list(self.bound) + [psi]:
            m = torch.empty_like(psi)
            self.op.apply(_lib.TDZ_MASS, v.contiguous(), m)
            mv.append(m)
        self._mv = mv
        self._ptrs = (C.c_void_p * len(mv))(*[m.data_ptr() for m in mv])
        self._out = torch.zeros(len(mv), dtype=torch.complex128, device=psi.device)

    def __call__(self, step: int, t: float, psi) -> None:
        import torch
        if self._mv is None:
            self._prepare(psi)
        s = torch.cuda.current_stream().cuda_stream
        norm, energy, dip = self.op.observables(psi)
        kin = self.op_kin.observables(psi)[1].real
        inv = self.op_inv.observables(psi)[1].real if self.op_inv is not None else self.inv_mass * norm
        k = len(self._mv)
        _lib.check(_lib.load().tdz_vec_mdot(self._ptrs, k, C.c_void_p(psi.data_ptr()), psi.numel(), _lib.TDZ_FP64,
                                            C.c_void_p(self._out.data_ptr()), C.c_void_p(s)))
        proj = self._out.cpu().numpy()
        e = np.zeros(3)
        if self.field is not None:
            fv = list(self.field(t))[:3]
            e[:len(fv)] = fv
        x = np.array([d.real for d in dip])
        sgn = -self.q
        e_int = sgn * float(e[:self.dim] @ x)
        self.file.record(
            t,
            dipoles=np.concatenate([e[:self.dim], self.q * x, np.zeros(self.dim)]),
            populations=np.abs(proj[:-1]) ** 2,
            energies=[kin, energy.real - kin, e_int, energy.real + e_int, inv, norm],
            autocorrelation=[proj[-1].real, proj[-1].imag])

    def close(self) -> None:
        self.file.close()


def write_surff(path: str, ts, amplitude: np.ndarray, flux: Optional[np.ndarray] = None, charge: float = -1.0,
                stride: int = 1, interior: bool = False, end_term: bool = False, end_nodes: int = 0,
                end_dp: float = 0.0) -> None:
    """The t-SURFF spectra file of ``ts`` (a ``TSurff``): datasets
    ``momenta`` (n_k x d), ``amplitude`` (n_k x 2: Re, Im of b(k)), ``pes``
    (|b|^2), ``amplitude_flux`` (the surface-flux part alone, with an
    interior or end term), ``k_x`` ... and ``pes_grid`` (the spectrum on the
    grid, k_x slowest); root attributes final_time, radius, exterior_mass,
    exterior_potential, charge, stride, n_surface_points, n_samples,
    interior, end_term, end_term_nodes, end_term_dp and A_final (d values),
    as in ``src/tsurff.cpp:1018-1057``. ``amplitude`` is the total spectrum
    (flux plus interior or end term)."""
    info = np.zeros(8)
    _lib.check(_lib.load().tdz_tsurff_info(ts.handle, _lib.dptr(info)))
    d = int(info[7])
    nk = [int(n) for n in ts.nk]
    axes = [np.asarray(a, dtype=np.float64) for a in ts.k_axes()]
    amp = np.asarray(amplitude, dtype=np.complex128).reshape(-1)
    if amp.size != int(np.prod(nk)):
        raise ValueError("amplitude has the wrong number of momenta")
    grids = np.meshgrid(*axes, indexing="ij")
    momenta = np.stack([g.reshape(-1) for g in grids], axis=1)
    pes = np.abs(amp) ** 2
    ds = {"momenta": momenta, "amplitude": np.stack([amp.real, amp.imag], axis=1), "pes": pes}
    if flux is not None:
        f = np.asarray(flux, dtype=np.complex128).reshape(-1)
        ds["amplitude_flux"] = np.stack([f.real, f.imag], axis=1)
    for a, name in enumerate(("k_x", "k_y", "k_z")[:d]):
        ds[name] = axes[a]
    ds["pes_grid"] = pes.reshape(nk)
    volkov = ts.volkov()
    attrs = {"final_time": info[0], "radius": info[1], "exterior_mass": info[2], "exterior_potential": info[3],
             "charge": charge, "stride": float(stride), "n_surface_points": info[4], "n_samples": info[5],
             "interior": 1.0 if interior else 0.0, "end_term": 1.0 if end_term else 0.0,
             "end_term_nodes": float(end_nodes), "end_term_dp": float(end_dp), "A_final": volkov[:d]}
    write_h5(path, ds, attrs)
