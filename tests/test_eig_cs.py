"""The complex symmetric axis eigenbasis of the FDM preconditioner
(gen_eig_complex, csrc/eig_cs.cpp), on the host: for B-spline axis operators
with the Manolopoulos absorbing layer, S = K/2 - i W against the overlap M
(assembled by the oracle), V^T M V = I and V^T S V = diag(lam) hold to
rounding, including the axes whose two mirror-image layers give pairs of
equal eigenvalues (60 elements of degree 4 on [-20, 20]). Built from the
library source with the host compiler; skipped without one."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import bspline as ob
from oracle import operators as oo

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    cuda_inc = None
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if cand and os.path.isfile(os.path.join(cand, "include", "cuda_runtime.h")):
            cuda_inc = os.path.join(cand, "include")
    if cuda_inc is None:
        pytest.skip("CUDA headers not found")
    exe = str(tmp_path_factory.mktemp("eig") / "eig_cs_check")
    csrc = os.path.join(ROOT, "tdsez_gb300", "csrc")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", csrc, "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                    os.path.join(HERE, "native", "eig_cs_check.cpp"), os.path.join(csrc, "eig_cs.cpp"), "-o", exe],
                   check=True)
    return exe


def _axis(p, L, nel, kmin, tmp_path):
    S = ob.Space([ob.Axis(ob.uniform_knots(nel, -L, L, p), p, p + 2)])
    A = oo.Assembled(S, oo.Physics(dim=1, cap_kmin=kmin, bounds=[(-L, L)], coupled=(0,)))
    M, H = A.M.toarray(), A.H_total().toarray()
    n = len(M)
    path = tmp_path / "band.txt"
    with open(path, "w") as f:
        f.write(f"{n} {p}\n")
        for i in range(n):
            for o in range(2 * p + 1):
                j = i - p + o
                m = M[i, j] if 0 <= j < n else 0.0
                h = H[i, j] if 0 <= j < n else 0.0
                f.write(f"{float(m)!r} {float(h.real)!r} {float(h.imag)!r}\n")
    return str(path), H, M


@pytest.mark.parametrize("p,L,nel,kmin", [(3, 18.0, 18, 1.0), (4, 20.0, 60, 1.0), (5, 20.0, 40, 1.0),
                                          (3, 60.0, 120, 0.8)])
def test_complex_axis_eigenbasis(checker, tmp_path, p, L, nel, kmin):
    path, H, M = _axis(p, L, nel, kmin, tmp_path)
    out = subprocess.run([checker, path], check=True, capture_output=True, text=True).stdout.split()
    ok, es, em = int(out[0]), float(out[1]), float(out[2])
    assert ok == 1
    assert es < 1e-11 and em < 1e-9, (es, em)
    # the mirror-image pairs are there: eigenvalues equal to rounding
    lam = np.linalg.eigvals(np.linalg.solve(M, H))
    d = np.abs(lam[:, None] - lam[None, :]) + np.eye(len(lam)) * 1e9
    if nel == 60:
        assert d.min() < 1e-9 * np.abs(lam).max()
