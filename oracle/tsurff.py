"""Oracle (test infrastructure only): t-SURFF surface flux of
``src/tsurff.cpp`` on the momentum grid.

* surface points: the Gauss points of every knot span clipped to [-R, R] on
  each tangential axis, faces x_a = +-R (``tsurff.cpp:112-137,148-176``);
* trace: psi and (1/m) d_n psi at each point (``tsurff.cpp:220-243``);
* Volkov integrals A' = -s E, B' = A, C' = |A|^2/2m + V0 by classical RK4 on
  substeps of at most TimeStep/2 (``tsurff.cpp:395-428``);
* flux per momentum (``FluxList``, ``tsurff.cpp:536-559``; the grid path
  ``FluxGrid`` ``:478-534`` is the same sum factorised by axis);
* trapezoid accumulation over samples (``AddFlux``, ``tsurff.cpp:439-469``);
* the end term (``EndTerm``, ``tsurff.cpp:650-976``) with one direct sparse
  solve per energy node in place of the reference's multi-shift Arnoldi.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse.linalg as sla

from .bspline import Space, find_span, ders_basis, gauss_legendre


class OracleTSurff:
    def __init__(self, space: Space, R: float, kgrid, mass: float, V0: float, sign: float,
                 field, dt: float, nq: int = 0, inv_mass_at=None):
        self.space = space
        self.dim = space.dim
        self.R = R
        self.mass = mass
        self.V0 = V0
        self.sign = sign
        self.field = field          # t -> E_a(t), length dim (0 on uncoupled axes)
        self.dt = dt
        nq = nq or space.axes[0].nq
        gx, gw = gauss_legendre(nq)
        self.nodes, self.weights = [], []
        for d in range(3):
            if d >= self.dim:
                self.nodes.append(np.array([0.0]))
                self.weights.append(np.array([1.0]))
                continue
            U = space.axes[d].knots
            xs, ws = [], []
            for j in range(len(U) - 1):
                lo, hi = max(U[j], -R), min(U[j + 1], R)
                if hi <= lo:
                    continue
                for k in range(nq):
                    xs.append(0.5 * (lo + hi) + 0.5 * (hi - lo) * gx[k])
                    ws.append(0.5 * (hi - lo) * gw[k])
            self.nodes.append(np.array(xs))
            self.weights.append(np.array(ws))
        # surface points and trace rows
        self.points = []    # (x[3], w, face, invMass)
        rows_v, rows_n = [], []
        for a in range(self.dim):
            for s in range(2):
                sigma = 1.0 if s else -1.0
                b = 1 if a == 0 else 0
                c = 1 if a == 2 else 2
                for ib, xb in enumerate(self.nodes[b]):
                    for ic, xc in enumerate(self.nodes[c]):
                        x = [0.0, 0.0, 0.0]
                        x[a] = sigma * R
                        x[b] = xb
                        x[c] = xc
                        w = self.weights[b][ib] * self.weights[c][ic]
                        im = 1.0 / mass if inv_mass_at is None else inv_mass_at(*x)
                        v, n = self._trace_row(x, a, sigma)
                        self.points.append((np.array(x), w, 2 * a + s, im))
                        rows_v.append(v)
                        rows_n.append(n * im)
        self.Tv = np.array(rows_v)
        self.Tn = np.array(rows_n)
        self.A = np.zeros(3)
        self.B = np.zeros(3)
        self.C = 0.0
        self.vt = 0.0
        self.prev = None
        self.prevT = 0.0

    def _trace_row(self, x, a, sigma):
        """Dense rows: value and normal derivative of every basis function."""
        sp_ = self.space
        vals, ders = [], []
        for d in range(self.dim):
            ax = sp_.axes[d]
            s = find_span(ax.knots, ax.p, ax.n, x[d])
            D = ders_basis(ax.knots, ax.p, s, x[d], 1)
            v = np.zeros(ax.n)
            dv = np.zeros(ax.n)
            v[s - ax.p:s + 1] = D[0]
            dv[s - ax.p:s + 1] = D[1]
            vals.append(v)
            ders.append(dv)
        V = vals[-1]
        N = ders[-1] if a == self.dim - 1 else vals[-1]
        for d in reversed(range(self.dim - 1)):
            V = np.kron(V, vals[d])
            N = np.kron(N, ders[d] if a == d else vals[d])
        return V, sigma * N

    def advance_volkov(self, t):
        h = t - self.vt
        if h <= 0:
            return
        n = max(1, int(math.ceil(h / (0.5 * self.dt) - 1e-9)))
        dt = h / n
        s, m, V0 = self.sign, self.mass, self.V0

        def f(tt, y):
            E = self.field(tt)
            dy = np.zeros(7)
            for d in range(3):
                dy[d] = -s * E[d] if d < self.dim else 0.0
                dy[3 + d] = y[d]
            dy[6] = (y[0] ** 2 + y[1] ** 2 + y[2] ** 2) / (2 * m) + V0
            return dy
        y = np.concatenate([self.A, self.B, [self.C]])
        for i in range(n):
            t0 = self.vt + i * dt
            k1 = f(t0, y)
            k2 = f(t0 + 0.5 * dt, y + 0.5 * dt * k1)
            k3 = f(t0 + 0.5 * dt, y + 0.5 * dt * k2)
            k4 = f(t0 + dt, y + dt * k3)
            y = y + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        self.A, self.B, self.C = y[:3].copy(), y[3:6].copy(), float(y[6])
        self.vt = t

    def flux(self, psi, kgrid):
        """Flux of psi at every momentum of the grid (list of per-axis arrays)."""
        v = self.Tv @ psi
        dn = self.Tn @ psi
        ks = [np.asarray(kgrid[d]) if d < self.dim else np.array([0.0]) for d in range(3)]
        K = np.stack(np.meshgrid(*ks, indexing="ij"), axis=-1).reshape(-1, 3)
        norm = (2 * math.pi) ** (-0.5 * self.dim)
        X = np.array([pt[0] for pt in self.points])                  # surface points (P, 3)
        W = np.array([pt[1] for pt in self.points])
        axis = np.array([pt[2] // 2 for pt in self.points])
        sigma = np.array([1.0 if pt[2] % 2 else -1.0 for pt in self.points])
        im = np.array([pt[3] for pt in self.points])
        out = np.zeros(len(K), dtype=np.complex128)
        for i0 in range(0, len(K), 256):            # blocks of momenta: every point at once
            k = K[i0:i0 + 256]
            phi = self.C + np.sum(self.vt * k * k / (2 * self.mass) + k * self.B / self.mass, axis=1)
            kA = k + self.A
            chi = W * np.exp(1j * (phi[:, None] - kA @ X.T))
            term = -dn[None, :] - 1j * (sigma * im)[None, :] * kA[:, axis] * v[None, :]
            out[i0:i0 + 256] = 0.5j * norm * np.sum(chi * term, axis=1)
        return out

    def add_flux(self, t, psi, kgrid, amp):
        self.advance_volkov(t)
        cur = self.flux(psi, kgrid)
        if self.prev is not None:
            amp += 0.5 * (t - self.prevT) * (self.prev + cur)
        self.prev = cur
        self.prevT = t
        return amp

    def interior(self, psi, kgrid):
        """Projection of psi(T) inside the box |x_d| < R onto the Volkov states
        at the last sample time (the SurffInterior term of tdsez_tsurff.hpp,
        ``Interior``/``Project``, ``src/tsurff.cpp:565-639``): adding it makes
        the spectrum exact for any final time."""
        sp_ = self.space
        ks = [np.asarray(kgrid[d]) for d in range(self.dim)]
        out = None
        # separable: psi values on the tensor grid of in-box Gauss points
        pts, wts, Bs = [], [], []
        for d in range(self.dim):
            ax = sp_.axes[d]
            xs, ws = self.nodes[d], self.weights[d]
            Bm = np.zeros((len(xs), ax.n))
            for i, x in enumerate(xs):
                s = find_span(ax.knots, ax.p, ax.n, x)
                Bm[i, s - ax.p:s + 1] = ders_basis(ax.knots, ax.p, s, x, 0)[0]
            pts.append(xs)
            wts.append(ws)
            Bs.append(Bm)
        G = psi.reshape(self.space.shape)
        for d in range(self.dim):       # contract axis d (x is the last array axis)
            G = np.moveaxis(np.tensordot(Bs[d], np.moveaxis(G, self.dim - 1 - d, 0), axes=(1, 0)),
                            0, self.dim - 1 - d)
        # integrate chi^* psi: factorised over axes
        for d in range(self.dim):
            E = np.exp(-1j * np.outer(ks[d] + self.A[d], pts[d])) * wts[d][None, :]
            G = np.moveaxis(np.tensordot(E, np.moveaxis(G, self.dim - 1 - d, 0), axes=(1, 0)),
                            0, self.dim - 1 - d)
        K = np.meshgrid(*reversed(ks), indexing="ij")   # shaped like G (slowest axis first)
        phi = self.C
        for d in range(self.dim):
            kd = K[self.dim - 1 - d]
            phi = phi + self.vt * kd * kd / (2 * self.mass) + kd * self.B[d] / self.mass
        out = (2 * math.pi) ** (-0.5 * self.dim) * np.exp(1j * phi) * G
        return np.moveaxis(out, list(range(self.dim)), list(reversed(range(self.dim)))).reshape(-1)


# --------------------------------------------------------------------------
# End term (SurffEndTerm = 1, ``src/tsurff.cpp:650-976``)
# --------------------------------------------------------------------------

def end_nodes(pmin, pmax, split, dp_in, dp_out):
    """Energy nodes in p = |k + A(T)| (``tsurff.cpp:700-723``): spacing dp_in
    on [pmin, split], dp_out on [split, pmax], midpoints added until there
    are four."""
    if not pmax > pmin:
        return np.array([pmin])
    node = []

    def segment(a, b, dp):
        # the last node is b itself: one rounding below it would open a second
        # segment with a node next to it (Lagrange weights over the difference)
        if not b > a:
            return
        cnt = max(1, int(math.ceil((b - a) / dp - 1e-9)))
        for i in range(0 if not node else 1, cnt + 1):
            node.append(b if i == cnt else a + (b - a) * i / cnt)
    segment(pmin, split, dp_in)
    segment(node[-1] if node else pmin, pmax, dp_out)
    while len(node) < 4:
        finer = []
        for a, b in zip(node[:-1], node[1:]):
            finer += [a, 0.5 * (a + b)]
        node = finer + [node[-1]]
    return np.array(node)


def lagrange_weights(node, p):
    """(first node, weights) of the four-point Lagrange interpolation in p
    around p (``tsurff.cpp:725-756``)."""
    nn = len(node)
    if nn == 1:
        return 0, np.array([1.0])
    m = min(nn, 4)
    below = int(np.searchsorted(node, p, side="right")) - 1
    j0 = max(0, min(nn - m, below - 1))
    w = np.ones(m)
    for a in range(m):
        for b in range(m):
            if b != a:
                w[a] *= (p - node[j0 + b]) / (node[j0 + a] - node[j0 + b])
    return j0, w


def end_term(ts: OracleTSurff, psi, M, H, kgrid, cap_width=0.0, dp=0.0):
    """End-term amplitudes of ``ts`` after its last sample (time T, Volkov
    state at T): per energy node E_j = p_j^2/2m + V0 the direct sparse solve
    of (E_j M - H) phi_j = i M psi(T) (H with the CAP), the flux of phi_j at
    T on every momentum, combined with the Lagrange weights of each momentum.
    Returns (amplitudes, nodes)."""
    ks = [np.asarray(kgrid[d]) if d < ts.dim else np.array([0.0]) for d in range(3)]
    K = np.stack(np.meshgrid(*ks, indexing="ij"), axis=-1).reshape(-1, 3)
    pk = np.linalg.norm(K + ts.A[None, :], axis=1)
    dk = min([(k[-1] - k[0]) / (len(k) - 1) for k in ks[:ts.dim] if len(k) > 1] or [np.inf])
    L = max(max(abs(a.knots[0]), abs(a.knots[-1])) for a in ts.space.axes)
    sd = math.sqrt(ts.dim)
    kcap = 6.555 / cap_width if cap_width > 0 else 0.0
    dp_out = dp if dp > 0 else min(dk, 0.25 / (ts.R * sd))
    dp_in = dp if dp > 0 else min(dp_out, 0.25 / (L * sd))
    split = min(max(2 * kcap, pk.min()), pk.max())
    node = end_nodes(pk.min(), pk.max(), split, dp_in, dp_out)
    W = np.zeros((len(node), len(K)))
    for q, p in enumerate(pk):
        j0, w = lagrange_weights(node, p)
        W[j0:j0 + len(w), q] = w
    b = 1j * (M @ psi)
    amp = np.zeros(len(K), dtype=np.complex128)
    for j, p in enumerate(node):
        E = p * p / (2 * ts.mass) + ts.V0
        phi = sla.splu((E * M - H).astype(np.complex128).tocsc()).solve(b)
        amp += W[j] * ts.flux(phi, kgrid)
    return amp, node
