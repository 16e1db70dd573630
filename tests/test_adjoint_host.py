"""The reverse-mode far-pair derivatives of the adjoint (adjoint.cuh),
compiled for the host: the vertex gradient of Re sum C0 H0 + C1 H1 over the
nine (Qa, Qb) choices (PanelPanelInteractions.cc:108-201, 6x6 rule) against
central differences of the forward moments, and the per-slot partial sums
(which carry the edge-length factors) against direct sums."""
import os
import subprocess
import tempfile

import pytest

from test_ffmath_host import _nvcc

HERE = os.path.dirname(os.path.abspath(__file__))


def test_far_pair_vjp_against_central_differences():
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "adjcheck")
        subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-ffp-contract=off",
                        "-o", exe, os.path.join(HERE, "adjoint_check.cu")], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    vals = dict(zip(out[0::2], map(float, out[1::2])))
    # central differences with h = 1e-5 on panels of size ~0.3: ~1e-10
    assert vals["grad"] < 1e-8, vals
    assert vals["slot"] < 1e-12, vals
