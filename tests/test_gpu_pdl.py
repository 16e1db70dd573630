"""Programmatic dependent launch changes when the LU's kernels start, not
what they compute: the complex-FP32 factorisation with the launch attribute
(default) and without it (GBEM_PDL=0, read once per process, so each variant
runs in its own process) must be bit-identical."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from gbem import C64, RWGGeometry, mesh
from gbem.api import HMatrix, Material
V, P = mesh.icosphere(3)
G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25)}])
M = HMatrix(G, C64)
rng = np.random.default_rng(11)
N = M.N
A = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
M.set(A)
assert M.LUFactorize() == 0
np.save(sys.argv[2], M.numpy())
np.save(sys.argv[3], np.asarray(M.ipiv))
"""


def _factor(tmp_path, tag, env_extra):
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ)
    env.update(env_extra)
    lu, piv = tmp_path / ("lu_%s.npy" % tag), tmp_path / ("piv_%s.npy" % tag)
    subprocess.run([sys.executable, "-c", _CHILD, os.path.join(repo, "scuff-em_gb300"), str(lu), str(piv)],
                   env=env, check=True, timeout=600)
    return np.load(lu), np.load(piv)


def test_programmatic_dependent_launch_is_bit_identical(tmp_path):
    # N = 3840: recursive panels with cluster leaves, tensor-core updates; the
    # tuned shapes are fixed so both processes run the same kernels
    fixed = {"GBEM_LU_PANEL": "256", "GBEM_LU_LEAF_THREADS": "512"}
    lu1, p1 = _factor(tmp_path, "pdl", fixed)
    lu0, p0 = _factor(tmp_path, "nopdl", dict(fixed, GBEM_PDL="0"))
    assert np.array_equal(p1, p0)
    assert np.ascontiguousarray(lu1).tobytes() == np.ascontiguousarray(lu0).tobytes()
