"""Oracle (test infrastructure only): the assembled-matrix operators of TDSE-Z
in FP64, and their Kronecker factorisation.

The assembled path restates the per-quadrature-point element arithmetic of
``TDSEZFormHam`` (``src/assembly/assembly.cpp:703-864``):

    H_ab = sum_q w_q [ 1/(2 m(x_q)) grad B_a . grad B_b + s V(x_q) B_a B_b ]
    M_ab = sum_q w_q B_a B_b

with s = -Charge (``include/tdsez_parser.hpp:92-105``), the dipoles
D_a = int x_a B B, and the Manolopoulos CAP of ``TDSEZformCap``
(``src/assembly/assembly.cpp:1945-1989``, profile ``:170-208``, layer width
``:1892-1895``, mass scale ``:1897-1906``):

    CAP = -i int W(r)/m B B,  W(r) = sum_d W_d(x_d).

The tensor Gauss rule is the union of the element rules, so the quadrature
sums are written as sparse products B^T diag(w f) B of the tensor basis
tables; they are the element loop with a different summation order.

Homogeneous Dirichlet walls follow ``TDSEZCompOperatorsDirichlet``
(``src/assembly/assembly.cpp:407-479,589-632``): wall rows and columns are
removed from H and M and each wall DoF gets, from every element that holds
it, ratio*mDiag on the H diagonal and mDiag on the M diagonal (ratio and
mDiag over the element's free DoFs); dipoles and CAP lose the wall rows and
columns (``TDSEZZeroDirichletRows(A, 0)``, ``src/assembler_class.cpp:270``).
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np
import scipy.sparse as sp

from .bspline import Axis, Space


# --------------------------------------------------------------------------
# Manolopoulos CAP
# --------------------------------------------------------------------------

MA_C = 2.62206


def cap_width(kmin: float) -> float:
    """Layer width c / (2 delta kmin), delta = 0.2 (``assembly.cpp:1892-1895``)."""
    return MA_C / (2.0 * 0.2 * kmin)


def manolopoulos_profile(u: float, width: float, kmin: float) -> float:
    """W at layer coordinate u in [0, width) (``assembly.cpp:170-208``)."""
    c = MA_C
    c3 = c ** 3
    a = 1.0 - 16.0 / c3
    b = (1.0 - 17.0 / c3) / (c * c)
    emin = 0.5 * kmin * kmin
    rcap = width - c / (2.0 * 0.2 * kmin)
    au = abs(u)
    if au <= rcap:
        return 0.0
    r = c * ((au - rcap) / (width - rcap))
    if au >= width:
        r = c * (1.0 - np.finfo(np.float64).eps)
    return emin * (a * r - b * r ** 3 + 4.0 / (c - r) ** 2 - 4.0 / (c + r) ** 2)


def cap_axis_profile(x: float, lo: float, hi: float, kmin: float) -> float:
    """One-axis CAP W_d(x) (``cap.cpp:31-36`` / ``assembly.cpp:1967-1976``)."""
    width = cap_width(kmin)
    s = min(x - lo, hi - x)
    if not (s < width):
        return 0.0
    return manolopoulos_profile(min(width - s, width * (1.0 - 1e-10)), width, kmin)


# --------------------------------------------------------------------------
# physics description
# --------------------------------------------------------------------------

@dataclass
class Physics:
    """Carrier and fields of one run.

    ``potential`` / ``inv_mass`` are callables of (x, y, z) (missing axes 0).
    ``pot_axis`` / ``mass_axis`` (optional) say that the function depends on
    that single axis only (layered structure), which the Kronecker form uses.
    ``pot_separable`` optionally lists per-axis 1D functions whose sum is V.
    """
    dim: int
    charge: float = -1.0
    potential: Callable = None
    inv_mass: Callable = None            # 1/m(r); None = 1
    mass_const: Optional[float] = 1.0    # set when the mass is constant
    pot_axis: Optional[int] = None
    mass_axis: Optional[int] = None
    pot_separable: Optional[Sequence[Optional[Callable]]] = None
    cap_kmin: Optional[float] = None     # None = no CAP
    bounds: Sequence[tuple] = ()          # (lo, hi) per axis
    coupled: Sequence[int] = (0,)         # polarisation: coupled axes
    dirichlet: bool = False

    @property
    def sign(self) -> float:
        """Carrier sign s = -Charge."""
        return -self.charge

    def V(self, *x):
        return 0.0 if self.potential is None else self.potential(*x)

    def minv(self, *x):
        if self.inv_mass is None:
            return 1.0 if self.mass_const is None else 1.0 / self.mass_const
        return self.inv_mass(*x)


def _kron(mats):
    """kron over axes given x first, producing the x-fastest ordering."""
    out = mats[-1]
    for m in reversed(mats[:-1]):
        out = sp.kron(out, m, format="csr")
    return out


def _eval_grid(f, coords, dim):
    pad = list(coords) + [np.zeros_like(coords[0])] * (3 - dim)
    return np.vectorize(f)(*pad[:3]) if f is not None else None


class Assembled:
    """H, M, D_a and CAP assembled by tensor quadrature (the reference's
    assembled AIJ path restated as scipy sparse matrices)."""

    def __init__(self, space: Space, phys: Physics):
        self.space = space
        self.phys = phys
        dim = space.dim
        B = [a.basis_matrix(0) for a in space.axes]
        dB = [a.basis_matrix(1) for a in space.axes]
        coords = [c.reshape(-1) for c in space.quad_coords()]
        w = space.quad_weights().reshape(-1)
        Bk = _kron(B)
        self.B = Bk
        s = phys.sign
        minv = _eval_grid(phys.minv, coords, dim)
        V = _eval_grid(phys.V, coords, dim) if phys.potential is not None else np.zeros_like(w)
        self.M = (Bk.T @ sp.diags(w) @ Bk).tocsr()
        K = None
        for a in range(dim):
            mats = [dB[d] if d == a else B[d] for d in range(dim)]
            Da = _kron(mats)
            term = Da.T @ sp.diags(0.5 * w * minv) @ Da
            K = term if K is None else K + term
        self.K = K.tocsr()
        self.V = (Bk.T @ sp.diags(w * s * V) @ Bk).tocsr()
        self.H = (self.K + self.V).tocsr()
        self.D = []
        for a in range(dim):
            self.D.append((Bk.T @ sp.diags(w * coords[a]) @ Bk).tocsr())
        self.CAP = None
        if phys.cap_kmin is not None:
            W = np.zeros_like(w)
            for d in range(dim):
                lo, hi = phys.bounds[d]
                W += np.vectorize(lambda x: cap_axis_profile(x, lo, hi, phys.cap_kmin))(coords[d])
            if phys.mass_const is not None:
                W *= 1.0 / phys.mass_const
            else:
                W *= minv
            self.CAP = (-1j * (Bk.T @ sp.diags(w * W) @ Bk)).tocsr()
        self.wall = None
        if phys.dirichlet:
            self._dirichlet(minv, V, w)

    # -- homogeneous Dirichlet (element rule) -------------------------------
    def _dirichlet(self, minv, V, w):
        sp_ = self.space
        dim = sp_.dim
        shape_x = [a.n for a in sp_.axes]
        nq_axis = [a.nel * a.nq for a in sp_.axes]
        minv = minv.reshape(list(reversed(nq_axis)))
        V = V.reshape(list(reversed(nq_axis)))
        s = self.phys.sign
        ndof = sp_.ndof
        hdiag = np.zeros(ndof)
        mdiag = np.zeros(ndof)
        wall_mask = np.zeros(ndof, dtype=bool)

        def gidx(loc):
            g, stride = 0, 1
            for d in range(dim):
                g += loc[d] * stride
                stride *= shape_x[d]
            return g

        for el in itertools.product(*[range(a.nel) for a in sp_.axes]):
            locs = list(itertools.product(*[range(a.p + 1) for a in sp_.axes]))
            # tensor tables on this element
            Ns = [sp_.axes[d].N[el[d]] for d in range(dim)]       # (nq, p+1)
            dNs = [sp_.axes[d].dN[el[d]] for d in range(dim)]
            ws = [sp_.axes[d].wq[el[d]] for d in range(dim)]
            qsl = tuple(slice(el[d] * sp_.axes[d].nq, (el[d] + 1) * sp_.axes[d].nq) for d in reversed(range(dim)))
            mi = minv[qsl]
            vv = V[qsl]
            Haa, Maa, gl, isw = [], [], [], []
            for loc in locs:
                # diagonal element entries
                val = [Ns[d][:, loc[d]] for d in range(dim)]
                der = [dNs[d][:, loc[d]] for d in range(dim)]
                wt = ws[0]
                prod0 = val[0] ** 2
                for d in range(1, dim):
                    wt = np.multiply.outer(ws[d], wt)
                    prod0 = np.multiply.outer(val[d] ** 2, prod0)
                m_aa = float((wt * prod0).sum())
                grad2 = 0.0
                for a in range(dim):
                    t = (der[0] if a == 0 else val[0]) ** 2
                    for d in range(1, dim):
                        t = np.multiply.outer((der[d] if a == d else val[d]) ** 2, t)
                    grad2 = grad2 + t
                h_aa = float((wt * (0.5 * mi * grad2 + s * vv * prod0)).sum())
                g = gidx([sp_.axes[d].offset[el[d]] + loc[d] for d in range(dim)])
                wallflag = any((sp_.axes[d].offset[el[d]] + loc[d]) in (0, shape_x[d] - 1) for d in range(dim))
                Haa.append(h_aa)
                Maa.append(m_aa)
                gl.append(g)
                isw.append(wallflag)
            if not any(isw):
                continue
            mD, ratio = 0.0, 1.0
            for h, m, wf in zip(Haa, Maa, isw):
                if wf:
                    continue
                if m > 0:
                    mD = max(mD, m)
                    ratio = max(ratio, abs(h) / m)
            if mD <= 0:
                mD = 1.0
            for g, wf in zip(gl, isw):
                if wf:
                    hdiag[g] += ratio * mD
                    mdiag[g] += mD
                    wall_mask[g] = True
        keep = sp.diags((~wall_mask).astype(np.float64))
        self.wall = wall_mask

        def pin(A, diag=None):
            A2 = (keep @ A @ keep).tocsr()
            if diag is not None:
                A2 = A2 + sp.diags(diag)
            return A2.tocsr()

        self.H = pin(self.H, hdiag)
        self.M = pin(self.M, mdiag)
        self.K = pin(self.K)
        self.V = pin(self.V)
        self.D = [pin(D) for D in self.D]
        if self.CAP is not None:
            self.CAP = pin(self.CAP)
        self.h_wall = hdiag
        self.m_wall = mdiag

    def H_total(self):
        """H with the CAP merged in (``src/propagator.cpp:55-64``)."""
        return self.H if self.CAP is None else (self.H + self.CAP).tocsr()

    def terms(self):
        """Field-term matrices of the coupled axes (``manager.cpp:1011-1018``)."""
        return [self.D[a] for a in self.phys.coupled if a < self.space.dim]


# --------------------------------------------------------------------------
# Kronecker factorisation (the form the GPU apply uses)
# --------------------------------------------------------------------------

@dataclass
class KronTerm:
    """coef * (A_z (x) A_y (x) A_x) with real 1D bands, x first in ``bands``."""
    coef: complex
    bands: list
    name: str = ""


def kron_terms(space: Space, phys: Physics, g: complex = 1.0, c=None, alpha: complex = 1.0,
               include_cap: bool = True):
    """Kronecker terms of A = alpha M + g (H + CAP + sum_a c_a D_a).

    Needs a separable physics: V = sum_d V_d(x_d) or V = V(x_a) for one axis,
    1/m constant or a function of one axis. Returns a list of KronTerm."""
    dim = space.dim
    ax = space.axes
    s = phys.sign
    Mb = [a.band() for a in ax]
    terms = [KronTerm(alpha, list(Mb), "M")]
    # kinetic
    if phys.mass_axis is None:
        minv = phys.minv(*([0.0] * 3))
        for a in range(dim):
            bands = list(Mb)
            bands[a] = ax[a].band(None, 1, 1)
            terms.append(KronTerm(g * 0.5 * minv, bands, f"K{a}"))
    else:
        ma = phys.mass_axis

        def minv_axis(x):
            pt = [0.0, 0.0, 0.0]
            pt[ma] = x
            return phys.minv(*pt)
        Mm = ax[ma].band(minv_axis)
        for a in range(dim):
            bands = list(Mb)
            if a == ma:
                bands[a] = ax[a].band(minv_axis, 1, 1)
            else:
                bands[a] = ax[a].band(None, 1, 1)
                bands[ma] = Mm
            terms.append(KronTerm(g * 0.5, bands, f"K{a}"))
    # potential
    if phys.potential is not None:
        if phys.pot_separable is not None:
            for d, f in enumerate(phys.pot_separable):
                if f is None:
                    continue
                bands = list(Mb)
                bands[d] = ax[d].band(f)
                terms.append(KronTerm(g * s, bands, f"V{d}"))
        elif phys.pot_axis is not None:
            pa = phys.pot_axis

            def v_axis(x):
                pt = [0.0, 0.0, 0.0]
                pt[pa] = x
                return phys.V(*pt)
            bands = list(Mb)
            bands[pa] = ax[pa].band(v_axis)
            terms.append(KronTerm(g * s, bands, f"V{pa}"))
        else:
            raise ValueError("potential is not separable")
    # CAP
    if include_cap and phys.cap_kmin is not None:
        if phys.mass_const is None:
            raise ValueError("separable CAP needs a constant mass")
        for d in range(dim):
            lo, hi = phys.bounds[d]
            bands = list(Mb)
            bands[d] = ax[d].band(lambda x: cap_axis_profile(x, lo, hi, phys.cap_kmin))
            terms.append(KronTerm(g * (-1j) / phys.mass_const, bands, f"W{d}"))
    # field terms
    if c is not None:
        for a, ca in zip(phys.coupled, c):
            if ca == 0:
                continue
            bands = list(Mb)
            bands[a] = ax[a].band(lambda x: x)
            terms.append(KronTerm(g * ca, bands, f"D{a}"))
    return terms


def band_apply_axis(A: np.ndarray, p: int, X: np.ndarray, axis: int) -> np.ndarray:
    """Contract a 1D band along one axis of an array shaped (.., n_axis, ..)."""
    n = A.shape[0]
    Xm = np.moveaxis(X, axis, -1)
    Y = np.zeros(Xm.shape, dtype=np.result_type(A, X))
    for k in range(-p, p + 1):
        lo, hi = max(0, -k), min(n, n - k)
        if hi <= lo:
            continue
        Y[..., lo:hi] += A[lo:hi, k + p] * Xm[..., lo + k:hi + k]
    return np.moveaxis(Y, -1, axis)


def kron_apply(space: Space, terms, x: np.ndarray) -> np.ndarray:
    """y = sum_t coef_t (A_z (x) A_y (x) A_x) x on the coefficient array
    (``src/tensorops.cpp:97-153``, one band contraction per axis)."""
    X = x.reshape(space.shape)
    Y = np.zeros(space.shape, dtype=np.complex128)
    dim = space.dim
    for t in terms:
        T = X
        for d in range(dim):
            T = band_apply_axis(t.bands[d], space.axes[d].p, T, dim - 1 - d)
        Y += t.coef * T
    return Y.reshape(-1)


def band_sparse(A: np.ndarray, p: int):
    """Sparse n x n matrix of a 1D band."""
    n = A.shape[0]
    rows, cols, vals = [], [], []
    for k in range(-p, p + 1):
        i = np.arange(max(0, -k), min(n, n - k))
        rows.append(i)
        cols.append(i + k)
        vals.append(A[i, k + p])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def kron_assemble(space: Space, terms):
    """Assembled sum_t coef_t (A_z (x) A_y (x) A_x) as a scipy sparse matrix."""
    out = None
    for t in terms:
        mats = [band_sparse(t.bands[d], space.axes[d].p) for d in range(space.dim)]
        m = t.coef * _kron(mats)
        out = m if out is None else out + m
    return out.tocsr()


def kron_operators(space: Space, phys: Physics):
    """M, H (+CAP) and the coupled dipoles of a separable physics, assembled
    from their Kronecker factors (equal to ``Assembled`` to rounding)."""
    M = kron_assemble(space, [t for t in kron_terms(space, phys, g=0.0, alpha=1.0) if t.name == "M"])
    H = kron_assemble(space, [t for t in kron_terms(space, phys, g=1.0, alpha=0.0) if t.name != "M"])
    D = []
    for a in phys.coupled:
        c = [1.0 if b == a else 0.0 for b in phys.coupled]
        D.append(kron_assemble(space, [t for t in kron_terms(space, phys, g=1.0, c=c, alpha=0.0)
                                       if t.name == f"D{a}"]))
    return M, H, D
