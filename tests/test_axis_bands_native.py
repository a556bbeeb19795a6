"""The 1D band matrices every operator is built from, as the library
computes them on the host (csrc/space.cpp; a small program linked against
libtdz.so, no GPU work), against the oracle's assembly by quadrature
(oracle/bspline.py): mass, stiffness, position and a potential band to
1e-13 of their largest entry, on uniform, graded and C0-interface knots of
degrees 2 to 5. Also the Galerkin coarse mass P^T M P of the multigrid
(csrc/mg_setup.cpp) equals the mass matrix assembled directly on the
coarsened knots, as it must for nested spline spaces (1e-13)."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import bspline as ob
from oracle import multigrid as om

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    from tdsez_gb300 import build
    build.build()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    cuda_inc = None
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if cand and os.path.isfile(os.path.join(cand, "include", "cuda_runtime.h")):
            cuda_inc = os.path.join(cand, "include")
    if cuda_inc is None:
        pytest.skip("CUDA headers not found")
    cuda_lib = os.path.join(os.path.dirname(cuda_inc), "lib64")
    exe = str(tmp_path_factory.mktemp("bands") / "axis_bands_check")
    pkg = os.path.join(ROOT, "tdsez_gb300")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(pkg, "csrc"), "-I", os.path.join(ROOT, "include"),
                    "-I", cuda_inc, os.path.join(HERE, "native", "axis_bands_check.cpp"), "-o", exe,
                    "-L", pkg, "-ltdz", "-Wl,-rpath," + pkg, "-L", cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib],
                   check=True)
    return exe


def _cases():
    out = []
    for p in (2, 3, 4, 5):
        nq = p + 1 + (p % 2)
        out.append((p, nq, ob.uniform_knots(14, -10.0, 10.0, p)))
        out.append((p, nq, ob.symexp_knots(-25.0, 25.0, 13, 0.9, p)))
        out.append((p, nq, ob.interface_knots(-12.0, 12.0, 15, p, [-4.0, 5.0])))
    return out


def _read(lines, k):
    name, rows, cols = lines[k].split()
    rows, cols = int(rows), int(cols)
    A = np.array([[float(v) for v in lines[k + 1 + i].split()] for i in range(rows)])
    return name, A, k + 1 + rows


def _oracle(ax, f=None, da=0, db=0):
    w = ax.wq.reshape(-1) * (1.0 if f is None else f(ax.xq.reshape(-1)))
    return (ax.basis_matrix(da).T @ sp.diags(w) @ ax.basis_matrix(db)).toarray()


def test_bands_match_the_oracle(checker):
    cases = _cases()
    text = "".join(f"{p} {nq} {len(U)} " + " ".join(repr(float(u)) for u in U) + "\n" for p, nq, U in cases)
    lines = subprocess.run([checker], input=text, capture_output=True, text=True, check=True).stdout.splitlines()
    k = 0
    for p, nq, U in cases:
        ax = ob.Axis(U, p, nq)
        ref = {"M": _oracle(ax), "S": _oracle(ax, None, 1, 1), "X": _oracle(ax, lambda x: x),
               "V": _oracle(ax, lambda x: x * x)}
        for name in ("M", "S", "X", "V"):
            got_name, A, k = _read(lines, k)
            assert got_name == name and A.shape == ref[name].shape
            err = np.abs(A - ref[name]).max() / np.abs(ref[name]).max()
            assert err < 1e-13, (p, len(U), name, err)
        name, G, k = _read(lines, k)
        C, _ = om.coarsen_knots(list(U))
        Mc = _oracle(ob.Axis(C, p, nq))
        assert name == "G" and G.shape == Mc.shape
        assert np.abs(G - Mc).max() / np.abs(Mc).max() < 1e-13, (p, len(U))
