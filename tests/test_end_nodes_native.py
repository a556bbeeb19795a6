"""The end term's energy nodes and four-point Lagrange weights as the
library computes them (tsurff_nodes.h, compiled for the host) against the
oracle's restatement (oracle/tsurff.py), on seeded random momentum ranges,
split points and spacings, including split = p_max and too few nodes."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import tsurff as ots

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("nodes") / "end_nodes_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "tdsez_gb300", "csrc"),
                    os.path.join(HERE, "native", "end_nodes_check.cpp"), "-o", exe], check=True)
    return exe


def test_nodes_and_weights_match_the_oracle(checker):
    rng = np.random.default_rng(2026)
    cases = []
    for i in range(60):
        pmin = rng.uniform(0.0, 1.0)
        pmax = pmin + rng.choice([rng.uniform(1e-3, 0.05), rng.uniform(0.1, 4.0)])
        split = rng.choice([pmax, pmin, rng.uniform(pmin, pmax), 2.0 * rng.uniform(0.2, 1.5)])
        split = float(min(max(split, pmin), pmax))
        pmin, pmax = float(pmin), float(pmax)
        dpi = float(rng.uniform(0.002, 0.1))
        dpo = float(rng.uniform(dpi, 0.3))
        ps = rng.uniform(pmin, pmax, size=7)
        cases.append((pmin, pmax, split, dpi, dpo, ps))
    # the oracle's own node-rule cases: split = p_max near an ulp, too few nodes, one node
    for pmax in (1.8411387545741371, 1.0 + 1e-13, 0.7 + 3 * 0.1):
        cases.append((0.3910663495531109, pmax, pmax, 0.25, 0.25, np.array([0.4, pmax])))
    cases.append((1.0, 1.1, 1.0, 1.0, 1.0, np.array([1.0, 1.05, 1.1])))
    cases.append((2.0, 2.0, 2.0, 0.1, 0.1, np.array([2.0])))
    text = "".join(f"{a!r} {b!r} {c!r} {d!r} {e!r} {len(ps)} " + " ".join(repr(float(p)) for p in ps) + "\n"
                   for a, b, c, d, e, ps in cases)
    out = subprocess.run([checker], input=text, capture_output=True, text=True, check=True).stdout.splitlines()
    k = 0
    for pmin, pmax, split, dpi, dpo, ps in cases:
        ref = ots.end_nodes(pmin, pmax, split, dpi, dpo)
        got = np.array([float(v) for v in out[k].split()[1:]])
        k += 1
        assert len(got) == len(ref) and np.allclose(got, ref, rtol=1e-15, atol=0)
        assert np.all(np.diff(got) > 0)
        for p in ps:
            j0r, wr = ots.lagrange_weights(ref, p)
            f = out[k].split()
            k += 1
            assert int(f[0]) == j0r
            assert np.allclose([float(v) for v in f[1:1 + len(wr)]], wr, rtol=1e-12, atol=1e-14)
