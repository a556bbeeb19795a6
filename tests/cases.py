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


@case("1d_cap_free")
def _c1c():
    """Free carrier in 1D with the absorbing layer (t-SURFF end term)."""
    p, nq = 4, 6
    return dict(knots=[ob.uniform_knots(60, -20.0, 20.0, p)], p=p, nq=nq, charge=-1.0, mass=1.0, V=[None],
                coupled=(0,), cap_kmin=0.5, bounds=[(-20.0, 20.0)])


@case("2d_cap_free")
def _c3c():
    """Free carrier in 2D with absorbing layers on both axes (t-SURFF end term)."""
    p, nq = 3, 5
    knots = [ob.uniform_knots(18, -18.0, 18.0, p), ob.uniform_knots(16, -16.0, 16.0, p)]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, V=[None, None], coupled=(0,), cap_kmin=1.0,
                bounds=[(-18.0, 18.0), (-16.0, 16.0)])


@case("3d_cap_free")
def _c3d_cap_free():
    """Free carrier in 3D with absorbing layers on every axis (t-SURFF end term)."""
    p, nq = 3, 4
    knots = [ob.uniform_knots(9, -12.0, 12.0, p), ob.uniform_knots(8, -11.0, 11.0, p),
             ob.uniform_knots(10, -13.0, 13.0, p)]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, V=[None, None, None], coupled=(2,), cap_kmin=1.2,
                bounds=[(-12.0, 12.0), (-11.0, 11.0), (-13.0, 13.0)])


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


def heterostructure_lines(p, nel_z):
    """3D heterostructure with short x / y axes and a long layered z axis: the
    FDM line solves along z take the two-thread (twisted) path once z has
    4 blocks of rows (32 rows for p = 3..5, 64 for p = 2)."""
    nq = p + 1
    br = [-9.0, 4.0]
    knots = [ob.uniform_knots(4, -8.0, 8.0, p), ob.uniform_knots(3, -7.0, 7.0, p),
             ob.interface_knots(-20.0, 20.0, nel_z, p, br)]
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


@case("2d_softcore")
def _c8():
    """The 2D soft-core Coulomb carrier of the 512^2 Pade(2,2) configuration,
    V = -1/sqrt(x^2 + y^2 + 1), with CAP and a field along x (small grid)."""
    p, nq = 4, 5
    knots = [ob.uniform_knots(14, -20.0, 20.0, p), ob.uniform_knots(13, -20.0, 20.0, p)]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, coupled=(0,), cap_kmin=1.0,
                bounds=[(-20.0, 20.0), (-20.0, 20.0)], soft=[(1.0, 0.0, 0.0, 0.0, 1.0)])


@case("3d_softcore")
def _c9():
    """The 3D soft-core carrier of the 192^3 Magnus-4 configuration,
    V = -1/sqrt(r^2 + 0.5), symmetric exponential knots with a knot at 0,
    field along z (small grid)."""
    p, nq = 4, 5
    knots = [ob.symexp_knots(-12.0, 12.0, 6, 0.9, p)] * 3
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, coupled=(2,), soft=[(1.0, 0.0, 0.0, 0.0, 0.5)])


@case("3d_two_centres_p3")
def _c10():
    """Two soft-core centres off the grid axes plus a separable confinement, p = 3."""
    p, nq = 3, 4
    knots = [ob.uniform_knots(7, -9.0, 9.0, p), ob.uniform_knots(6, -8.0, 8.0, p), ob.uniform_knots(8, -10.0, 10.0, p)]
    V = [lambda x: 0.005 * x * x, None, None]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, V=V, coupled=(0, 1, 2),
                soft=[(0.5, -1.0, 0.0, 0.0, 1.0), (0.7, 1.0, 0.5, -0.5, 0.8)])


@case("3d_softcore_tiles")
def _c11():
    """Two soft-core centres on a grid of several element tiles in x and y
    and two chunks along z (the tiled, z-streamed quadrature kernel), graded
    knots on x and z, p = 3."""
    p, nq = 3, 4
    knots = [ob.symexp_knots(-20.0, 20.0, 15, 0.9, p), ob.uniform_knots(12, -18.0, 18.0, p),
             ob.symexp_knots(-24.0, 24.0, 43, 0.9, p)]
    return dict(knots=knots, p=p, nq=nq, charge=-1.0, mass=1.0, coupled=(2,),
                soft=[(1.0, 0.3, -0.2, 0.1, 0.5), (0.5, -2.0, 1.0, 3.0, 1.0)])


def _soft_value(soft, r):
    v = 0.0
    for Z, cx, cy, cz, a in soft:
        d = (r[0] - cx, r[1] - cy, r[2] - cz)
        v -= Z / np.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2 + a)
    return v


def oracle_of(c):
    """Oracle Space, Physics, Assembled for a case dict."""
    S, ph = oracle_space_phys(c)
    return S, ph, oo.Assembled(S, ph)


def oracle_space_phys(c):
    """Oracle Space and Physics for a case dict, without assembling (large
    separable cases use the oracle's Kronecker apply instead)."""
    axes = [ob.Axis(k, c["p"], c["nq"]) for k in c["knots"]]
    S = ob.Space(axes)
    dim = S.dim
    Vs = list(c.get("V", [None] * dim)) + [None] * 3
    soft = c.get("soft", [])
    have_v = any(v is not None for v in Vs[:dim]) or bool(soft)

    def pot(x, y, z):
        r = (x, y, z)
        v = sum(Vs[d](r[d]) for d in range(dim) if Vs[d] is not None)
        if soft:   # 2D cases: the centres' z offset is irrelevant (r_z = 0, c_z = 0)
            v += _soft_value(soft, (x, y if dim > 1 else 0.0, z if dim > 2 else 0.0))
        return v
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
    return S, ph


def workload_case(nel, p=3):
    """The benchmark's 3D heterostructure (tdsez_gb300.workloads) at another
    element count, as a case dict: same box, layers, masses, potentials and
    field axis."""
    from tdsez_gb300.workloads import heterostructure
    w = heterostructure(nel=nel, p=p)
    return dict(knots=w.knots, p=w.p, nq=w.nq, charge=w.phys.charge, mass_axis=2, inv_mass=w.phys.inv_mass_fn,
                V=list(w.phys.potential), coupled=(2,)), w


def product_of(c):
    """Library Space and Operator for a case dict (needs libtdz.so)."""
    from tdsez_gb300.space import Space
    from tdsez_gb300.operators import Operator, Physics
    S = Space(c["knots"], c["p"], c["nq"])
    dim = S.dim
    ph = Physics(charge=c["charge"], mass=c.get("mass", 1.0), mass_axis=c.get("mass_axis"),
                 inv_mass_fn=c.get("inv_mass"), potential=list(c.get("V", [])), cap_kmin=c.get("cap_kmin"),
                 bounds=c.get("bounds", ()), coupled=c["coupled"], dirichlet=c.get("dirichlet", False),
                 softcore=c.get("soft", ()))
    return S, Operator(S, ph)
