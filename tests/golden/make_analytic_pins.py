"""Write analytic_pins.json: the closed forms and exact energies that the
reference's own tests assert (tests/test_analytic.py of the TDSE-Z tree).
The double-well and mass-step values are the reference's literal pins; the
remaining roots are recomputed here by the reference tests' transfer-matrix
method (brentq on the BDD matching conditions)."""
import json
import math
import os

import numpy as np
from scipy.optimize import brentq


def mass_step_dirichlet(m1, m2, nmin):
    def f(E):
        k1, k2 = np.sqrt(2 * m1 * E), np.sqrt(2 * m2 * E)
        return (k1 / m1) * np.cos(k1) * np.sin(k2) + (k2 / m2) * np.sin(k1) * np.cos(k2)
    Es = np.linspace(1e-6, 40.0, 40000)
    fs = f(Es)
    return [brentq(f, Es[i], Es[i + 1], xtol=1e-16, rtol=1e-15)
            for i in range(len(Es) - 1) if fs[i] * fs[i + 1] < 0][:nmin]


def layered_neumann(widths, masses, pots, nmin, emax):
    def f(E):
        u = np.array([1.0, 0.0])
        for w, m, V in zip(widths, masses, pots):
            q2 = 2.0 * m * (E - V)
            if q2 > 0:
                k = np.sqrt(q2)
                c, s = np.cos(k * w), np.sin(k * w)
                T = np.array([[c, m * s / k], [-k * s / m, c]])
            else:
                k = np.sqrt(-q2)
                c, s = np.cosh(k * w), np.sinh(k * w)
                T = np.array([[c, m * s / k], [k * s / m, c]])
            u = T @ u
            u /= np.max(np.abs(u))
        return u[1]
    Es = np.linspace(1e-6, emax, 20000)
    fs = np.array([f(E) for E in Es])
    return [brentq(f, Es[i], Es[i + 1], xtol=1e-16, rtol=1e-15)
            for i in range(len(Es) - 1) if fs[i] * fs[i + 1] < 0][:nmin]


pins = {
    "infinite_well": {"L": 10.0, "E": [n * n * math.pi ** 2 / 200.0 for n in range(1, 5)]},
    "double_quantum_well": {"E_meV": [40.6074468017, 43.4686725099], "hartree_mev": 27211.386},
    "mass_step": {
        "Dirichlet": {"E": mass_step_dirichlet(1.0, 4.0, 3)},
        "Neumann": {"E": [0.0] + layered_neumann([1.0, 1.0], [1.0, 4.0], [0.0, 0.0], 2, 10.0)},
    },
    "driven_oscillator": {"E0": 0.5, "omega": 0.6,
                          "x_of_t": "-E0/(1-omega^2) (cos(omega t) - cos t)"},
    "free_packet": {"pes": "prod_d (2 w^2/pi)^(1/2) exp(-2 w^2 (k_d - k0_d)^2)"},
}
assert abs(pins["mass_step"]["Dirichlet"]["E"][0] - 0.6615513245573471) < 1e-12
assert abs(pins["mass_step"]["Dirichlet"]["E"][1] - 1.9826989028677189) < 1e-12
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "analytic_pins.json")
json.dump(pins, open(out, "w"), indent=1)
print(out)
