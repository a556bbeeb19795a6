"""The multigrid hierarchy as the library builds it on the host (knot
coarsening and prolongation, csrc/mg_setup.cpp, called from a small program
linked against libtdz.so; no GPU work) against the oracle's restatement of
the reference's CoarsenKnots and Boehm Prolongation (src/multigrid.cpp:25-81,
oracle/multigrid.py): the same coarse knots and the same prolongation to
1e-12, on uniform, graded (symexp) and interface (C0) knot vectors of
degrees 2 to 5."""
import os
import shutil
import subprocess

import numpy as np
import pytest

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
    exe = str(tmp_path_factory.mktemp("mg") / "mg_hierarchy_check")
    pkg = os.path.join(ROOT, "tdsez_gb300")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(pkg, "csrc"), "-I", os.path.join(ROOT, "include"),
                    "-I", cuda_inc, os.path.join(HERE, "native", "mg_hierarchy_check.cpp"), "-o", exe,
                    "-L", pkg, "-ltdz", "-Wl,-rpath," + pkg, "-L", cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib],
                   check=True)
    return exe


def _knot_vectors():
    out = []
    for p in (2, 3, 4, 5):
        out.append((p, ob.uniform_knots(24, -20.0, 20.0, p)))
        out.append((p, ob.symexp_knots(-30.0, 30.0, 17, 0.9, p)))
        out.append((p, ob.interface_knots(-15.0, 15.0, 21, p, [-6.0, 3.0])))
    return out


def test_hierarchy_matches_the_oracle(checker):
    cases = _knot_vectors()
    text = "".join(f"{p} {len(U)} " + " ".join(repr(float(u)) for u in U) + "\n" for p, U in cases)
    lines = subprocess.run([checker], input=text, capture_output=True, text=True, check=True).stdout.splitlines()
    k = 0
    for p, U in cases:
        C_ref, dropped_ref = om.coarsen_knots(list(U))
        head = lines[k].split()
        k += 1
        C = np.array([float(v) for v in head[2:2 + int(head[0])]])
        assert int(head[1]) == int(dropped_ref) and np.array_equal(C, C_ref), (p, len(U))
        rows, cols, nnz = (int(v) for v in lines[k].split())
        k += 1
        P = np.zeros((rows, cols))
        for _ in range(nnz):
            r, c, v = lines[k].split()
            k += 1
            P[int(r), int(c)] = float(v)
        P_ref = om.prolongation(C_ref, np.asarray(U), p)
        assert P.shape == P_ref.shape
        assert np.abs(P - P_ref).max() < 1e-12, (p, len(U), np.abs(P - P_ref).max())
        # partition of unity: the coarse constant is the fine constant
        assert np.allclose(P.sum(axis=1), 1.0, atol=1e-12)
