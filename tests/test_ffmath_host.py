"""The float-float arithmetic of the mixed-precision far field (ffmath.cuh),
compiled for the host and checked against FP64 evaluations of the same sums:
e^{ix}, the 9+9 panel-pair moments and the H0/H1 combinations of
PanelPanelInteractions.cc:108-201 (GetPPIs_Cubature) for random far pairs.
The bound 1e-9 is what keeps the absorbed power of a weakly lossy sphere
within 1e-8 of the FP64 path (FP32 arithmetic gives ~1e-7 here and moves it
by ~1e-5)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return None


def test_ffmath_against_fp64():
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "ffcheck")
        subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-ffp-contract=off",
                        "-o", exe, os.path.join(HERE, "ffmath_check.cu")], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    vals = dict(zip(out[0::2], map(float, out[1::2])))
    assert vals["expi"] < 1e-10
    for key in ("mg", "mp", "h0", "h1"):
        assert vals[key] < 1e-9, (key, vals[key])
