"""The real axis eigenbasis of the fast-diagonalisation preconditioner
(gen_eig, csrc/fdm.cu: banded Cholesky of M, cyclic Jacobi on L^-1 S L^-T),
computed on the host by a small program linked against libtdz.so, against
the oracle's stiffness and mass matrices: V^T M V = I and V^T S V =
diag(lam) to 1e-12 of |lam|_max, and lam equal to scipy's generalised
symmetric eigenvalues to 1e-12 relative, up to the 163-function axes of the
heterostructure (p = 3, 160 elements)."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.linalg as la
import scipy.sparse as sp

from oracle import bspline as ob

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
    exe = str(tmp_path_factory.mktemp("eig") / "axis_eig_check")
    pkg = os.path.join(ROOT, "tdsez_gb300")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(pkg, "csrc"), "-I", os.path.join(ROOT, "include"),
                    "-I", cuda_inc, os.path.join(HERE, "native", "axis_eig_check.cpp"), "-o", exe,
                    "-L", pkg, "-ltdz", "-Wl,-rpath," + pkg, "-L", cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib],
                   check=True)
    return exe


def test_axis_eigenbasis(checker):
    cases = [(3, 4, ob.uniform_knots(160, -75.0, 75.0, 3)),
             (2, 3, ob.symexp_knots(-30.0, 30.0, 41, 0.9, 2)),
             (4, 5, ob.interface_knots(-20.0, 20.0, 37, 4, [-5.0, 6.0])),
             (5, 6, ob.uniform_knots(23, -8.0, 8.0, 5))]
    text = "".join(f"{p} {nq} {len(U)} " + " ".join(repr(float(u)) for u in U) + "\n" for p, nq, U in cases)
    lines = subprocess.run([checker], input=text, capture_output=True, text=True, check=True).stdout.splitlines()
    k = 0
    for p, nq, U in cases:
        ax = ob.Axis(U, p, nq)
        w = sp.diags(ax.wq.reshape(-1))
        M = (ax.basis_matrix(0).T @ w @ ax.basis_matrix(0)).toarray()
        S = (ax.basis_matrix(1).T @ w @ ax.basis_matrix(1)).toarray()
        n = int(lines[k])
        lam = np.array([float(v) for v in lines[k + 1].split()])
        V = np.array([[float(v) for v in lines[k + 2 + i].split()] for i in range(n)])
        k += 2 + n
        assert n == M.shape[0]
        scale = np.abs(lam).max()
        assert np.abs(V.T @ M @ V - np.eye(n)).max() < 1e-12
        assert np.abs(V.T @ S @ V - np.diag(lam)).max() < 1e-12 * scale
        ref = la.eigh(S, M, eigvals_only=True)
        assert np.abs(np.sort(lam) - ref).max() < 1e-12 * scale, (p, n)
