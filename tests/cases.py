"""Parity cases shared by the tests: the same space and physics built once
for the oracle (FP64 CPU restatement) and once for the GPU library."""
from __future__ import annotations

import numpy as np

from oracle import bspline as ob
from oracle import operators as oo


def _layered(breaks, values):
    def f(x):
        for b, v in zip(breaks, values):
            if x < b:
                return v
        return values[-1]
    return f


CASES = {}


def case(name):
    def deco(fn):
        CASES[name] = fn
        return fn
    return deco


@case("1d_dirichlet_ho")
def _c1():
    p, nq = 5, 6
    knots = [ob.uniform_knots(40, -20.0, 20.0, p)]
    V = [lambda x: 0.5 * x * x]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, V=V, coupled=(0,), dirichlet=True)


@case("1d_layered_mass")
def _c2():
    p, nq = 4, 6
    kn = ob.interface_knots(-30.0, 30.0, 29, p, [-5.0, 5.0])
    m = _layered([-5.0, 5.0], [0.0879, 0.067, 0.0879])
    V = [_layered([-5.0, 5.0], [0.00893, 0.0, 0.00893])]
    return dict(knots=[kn], p=p, nq=nq, charge=-1.0, mass_axis=0, inv_mass=lambda x: 1.0 / m(x), V=V,
                coupled=(0,))


@case("2d_cap_softcore_sep")
def _c3():
    p, nq = 4, 5
    knots = [ob.uniform_knots(12, -20.0, 20.0, p), ob.symexp_knots(-24.0, 24.0, 13, 0.9, p)]
    V = [lambda x: -0.3 / np.sqrt(x * x + 1.0), lambda y: 0.01 * y * y]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, V=V, coupled=(0,), cap_kmin=1.0,
                bounds=[(-20.0, 20.0), (-24.0, 24.0)])


@case("3d_heterostructure")
def _c4():
    p, nq = 3, 4
    br = [-6.0, 3.0]
    knots = [ob.uniform_knots(7, -10.0, 10.0, p), ob.uniform_knots(6, -9.0, 9.0, p),
             ob.interface_knots(-15.0, 15.0, 11, p, br)]
    m = _layered(br, [0.067, 0.092, 0.067])
    V = [None, None, _layered(br, [0.0, -0.2, 0.1])]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass_axis=2, inv_mass=lambda z: 1.0 / m(z), V=V,
                coupled=(2,))


@case("3d_const_mass_cap")
def _c5():
    p, nq = 4, 5
    knots = [ob.uniform_knots(6, -12.0, 12.0, p), ob.uniform_knots(5, -10.0, 10.0, p),
             ob.symexp_knots(-14.0, 14.0, 7, 0.9, p)]
    V = [lambda x: 0.05 * x * x, None, lambda z: -0.1 * np.exp(-z * z)]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=0.5, V=V, coupled=(0, 2), cap_kmin=1.2,
                bounds=[(-12.0, 12.0), (-10.0, 10.0), (-14.0, 14.0)])


@case("3d_p2_hole")
def _c6():
    p, nq = 2, 3
    knots = [ob.uniform_knots(9, -5.0, 5.0, p), ob.uniform_knots(8, -4.0, 4.0, p),
             ob.uniform_knots(10, -6.0, 6.0, p)]
    V = [lambda x: 0.2 * x, lambda y: 0.1 * y * y, None]
    return dict(knots=knots, p=p, nq=nq, charge=1.0, mass=2.0, V=V, coupled=(1,))


@case("3d_p5_sym")
def _c7():
    p, nq = 5, 6
    knots = [ob.symexp_knots(-8.0, 8.0, 6, 0.9, p), ob.uniform_knots(5, -6.0, 6.0, p),
             ob.uniform_knots(6, -7.0, 7.0, p)]
    V = [lambda x: 0.01 * x * x, lambda y: 0.01 * y * y, lambda z: 0.01 * z * z]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, V=V, coupled=(0, 1, 2))


def oracle_of(c):
    """Oracle Space, Physics, Assembled for a case dict."""
    axes = [ob.Axis(k, c["p"], c["nq"]) for k in c["knots"]]
    S = ob.Space(axes)
    dim = S.dim
    Vs = list(c.get("V", [None] * dim)) + [None] * 3
    have_v = any(v is not None for v in Vs[:dim])

    def pot(x, y, z):
        r = (x, y, z)
        return sum(Vs[d](r[d]) for d in range(dim) if Vs[d] is not None)
    ma = c.get("mass_axis")
    if ma is None:
        ph = oo.Physics(dim=dim, charge=c["charge"], potential=pot if have_v else None,
                        mass_const=c.get("mass", 1.0), pot_separable=[Vs[d] for d in range(dim)],
                        cap_kmin=c.get("cap_kmin"), bounds=c.get("bounds", ()), coupled=c["coupled"],
                        dirichlet=c.get("dirichlet", False))
    else:
        im = c["inv_mass"]

        def inv_mass(x, y, z):
            return im((x, y, z)[ma])
        ph = oo.Physics(dim=dim, charge=c["charge"], potential=pot if have_v else None, inv_mass=inv_mass,
                        mass_const=None, mass_axis=ma, pot_separable=[Vs[d] for d in range(dim)],
                        cap_kmin=c.get("cap_kmin"), bounds=c.get("bounds", ()), coupled=c["coupled"],
                        dirichlet=c.get("dirichlet", False))
    return S, ph, oo.Assembled(S, ph)


def product_of(c):
    """Library Space and Operator for a case dict (needs libtdz.so)."""
    from tdsez_gb300.space import Space
    from tdsez_gb300.operators import Operator, Physics
    S = Space(c["knots"], c["p"], c["nq"])
    dim = S.dim
    ph = Physics(charge=c["charge"], mass=c.get("mass", 1.0), mass_axis=c.get("mass_axis"),
                 inv_mass_fn=c.get("inv_mass"), potential=list(c.get("V", [])), cap_kmin=c.get("cap_kmin"),
                 bounds=c.get("bounds", ()), coupled=c["coupled"], dirichlet=c.get("dirichlet", False))
    return S, Operator(S, ph)
