"""Synthetic workloads with the shapes of the propagation benchmarks.

``heterostructure`` is the 3D layered structure of the Crank-Nicolson
steps/s metric: 160 x 160 x 320 elements of degree 3, five C0 interfaces
along z (layer widths drawn uniformly in [0.1, 0.3] of the box and
normalised, seed 20261203), piecewise V in {0.1, -0.2, 0} Ha and
m in {0.092, 0.067} per layer (barrier / well / spacer cycle), a field
along z with E0 drawn uniformly in [0.001, 0.01] (same seed), a sin^2
envelope over 6 cycles of omega = 0.057, and a Gaussian packet in the first
well. The box is [-150, 150]^2 x [-300, 300] a.u. (h = 1.875 a.u.) and the
step dt = 0.5 a.u.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, Sequence

import numpy as np

from .operators import MA_C, Physics
from .space import interface_knots, symexp_knots, uniform_knots

SEED = 20261203
V_CYCLE = (0.1, -0.2, 0.0)
M_CYCLE = (0.092, 0.067, 0.067)


@dataclass
class Workload:
    name: str
    knots: list
    p: int
    nq: int
    phys: Physics
    field: Callable[[float], Sequence[float]]
    dt: float
    packet: list          # per-axis callables for the initial state
    meta: dict


def _layers(L0: float, L1: float, nlayers: int, rng):
    w = rng.uniform(0.1, 0.3, nlayers)
    w = w / w.sum() * (L1 - L0)
    return list(L0 + np.cumsum(w)[:-1])


def heterostructure(nel=(160, 160, 320), p: int = 3, box=(150.0, 150.0, 300.0), dt: float = 0.5,
                    seed: int = SEED) -> Workload:
    rng = np.random.default_rng(seed)
    Lx, Ly, Lz = box
    breaks = _layers(-Lz, Lz, 6, rng)
    E0 = float(rng.uniform(0.001, 0.01))
    vals_v = [V_CYCLE[i % 3] for i in range(6)]
    vals_m = [M_CYCLE[i % 3] for i in range(6)]

    def layer(z):
        for i, b in enumerate(breaks):
            if z < b:
                return i
        return len(breaks)

    def vz(z):
        return vals_v[layer(z)]

    def inv_mz(z):
        return 1.0 / vals_m[layer(z)]

    knots = [uniform_knots(nel[0], -Lx, Lx, p), uniform_knots(nel[1], -Ly, Ly, p),
             interface_knots(-Lz, Lz, nel[2], p, breaks)]
    phys = Physics(charge=-1.0, mass_axis=2, inv_mass_fn=inv_mz, potential=[None, None, vz], coupled=(2,))
    omega, ncyc = 0.057, 6
    T = ncyc * 2 * math.pi / omega

    def field(t):
        env = math.sin(math.pi * t / T) ** 2 if 0 <= t <= T else 0.0
        return [E0 * env * math.cos(omega * t)]
    zc = 0.5 * (breaks[0] + breaks[1])        # centre of the first well
    w = 0.15 * (breaks[1] - breaks[0])
    packet = [lambda x: np.exp(-x * x / (2 * 40.0 ** 2)), lambda y: np.exp(-y * y / (2 * 40.0 ** 2)),
              lambda z: np.exp(-(z - zc) ** 2 / (2 * w ** 2))]
    meta = {"elements": list(nel), "degree": p, "box_au": [2 * Lx, 2 * Ly, 2 * Lz], "interfaces": breaks,
            "V_layers": vals_v, "m_layers": vals_m, "E0": E0, "omega": omega, "cycles": ncyc, "dt": dt}
    return Workload("heterostructure", knots, p, p + 1, phys, field, dt, packet, meta)


def _pulse(E0: float, omega: float, cycles: int, axis_count: int, axis: int, cep: float = 0.0):
    """sin^2 envelope over `cycles` cycles of cos(omega t + cep) on one axis."""
    T = cycles * 2 * math.pi / omega

    def field(t):
        env = math.sin(math.pi * t / T) ** 2 if 0 <= t <= T else 0.0
        e = [0.0] * axis_count
        e[axis] = E0 * env * math.cos(omega * t + cep)
        return e
    return field, T


def softcore2d(nel: int = 512, p: int = 4, L: float = 100.0, cap_width: float = 20.0, dt: float = 0.02,
               cap: bool = True) -> Workload:
    """2D soft-core hydrogen, V = -1/sqrt(x^2 + y^2 + 1) on [-L, L]^2 with nel^2
    elements of degree p (Q = p + 1 Gauss points), a Manolopoulos CAP of
    width `cap_width` on every wall (kmin = c / (2 delta width), the
    reference's CAPWidth input), a 4-cycle sin^2 pulse along x with
    E0 = 0.05, omega = 0.057, Pade(2,2) with dt = 0.02 and t-SURFF on the
    square |x_d| = 80 (the reference's t-SURFF surface; no circle there)."""
    knots = [uniform_knots(nel, -L, L, p)] * 2
    kmin = MA_C / (2.0 * 0.2 * cap_width)
    phys = Physics(charge=-1.0, mass=1.0, coupled=(0,), softcore=[(1.0, 0.0, 0.0, 0.0, 1.0)],
                   cap_kmin=kmin if cap else None, bounds=[(-L, L), (-L, L)] if cap else ())
    field, T = _pulse(0.05, 0.057, 4, 1, 0)
    meta = {"elements": [nel, nel], "degree": p, "box_au": [2 * L, 2 * L], "cap_width": cap_width if cap else 0.0,
            "E0": 0.05, "omega": 0.057, "cycles": 4, "T": T, "dt": dt, "surff_radius": 80.0}
    return Workload("softcore2d", knots, p, p + 1, phys, field, dt,
                    [lambda x: np.exp(-x * x / 2.0)] * 2, meta)


def softcore3d(nel: int = 192, p: int = 4, L: float = 60.0, alpha: float = 0.9, dt: float = 0.02) -> Workload:
    """3D soft-core atom, V = -1/sqrt(r^2 + 0.5) on [-L, L]^3 with nel^3
    elements of degree p (Q = p + 1), symmetric exponential knots with
    KnotAlpha 0.9 (even nel puts a knot at 0), a 6-cycle sin^2 pulse along z
    with E0 = 0.053, omega = 0.057, Magnus-4 with dt = 0.02."""
    knots = [symexp_knots(-L, L, nel, alpha, p)] * 3
    phys = Physics(charge=-1.0, mass=1.0, coupled=(2,), softcore=[(1.0, 0.0, 0.0, 0.0, 0.5)])
    field, T = _pulse(0.053, 0.057, 6, 1, 0)
    meta = {"elements": [nel] * 3, "degree": p, "box_au": [2 * L] * 3, "knot_alpha": alpha, "E0": 0.053,
            "omega": 0.057, "cycles": 6, "T": T, "dt": dt}
    # the hydrogen-like 1s shape exp(-r) is not separable; exp(-x^2/2) per axis is
    return Workload("softcore3d", knots, p, p + 1, phys, field, dt, [lambda x: np.exp(-x * x / 2.0)] * 3, meta)

