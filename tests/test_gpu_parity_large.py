"""The BEM matrix at the benchmark's own size (dielectric icosphere s=4,
5120 panels, PMCHWT N = 15360, eps = 2.25+0.01i, kR = 2) against the oracle,
column by column: 32 seeded whole columns, each holding the self pair, ~40
near panel pairs and the far field of one basis function against every
other.  The oracle's columns equal its full assembly entry for entry
(tests/test_oracle.py), so this pins the N = 15360 matrix itself, in both
the plain FP64 form and the mixed form (float-float far field rounded once to
complex64)."""
import numpy as np
import pytest

from helpers import device_columns

pytestmark = pytest.mark.gpu

EPS = 2.25 + 0.01j
W = 2.0


@pytest.fixture(scope="module")
def setup():
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    from oracle import oracle
    V, P = mesh.icosphere(4)
    G = RWGGeometry([{"V": V, "P": P, "material": Material(EPS)}])
    N = G.TotalBFs
    assert N == 15360
    rng = np.random.default_rng(0)
    cols = np.unique(np.concatenate([[0, 1, N - 2, N - 1], rng.choice(N, 28, replace=False)]))
    Mo = oracle.assemble_cols([oracle.Surface(V, P)], [(0, 1)], [False], W, [1.0, EPS], [1.0, 1.0], cols)
    return G, cols, Mo


def test_fp64_matrix_columns_match_oracle(setup):
    G, cols, Mo = setup
    M = G.AssembleBEMMatrix(W)
    Mc = device_columns(M, cols)
    del M
    scale = np.abs(Mo).max()
    err = np.abs(Mc - Mo).max() / scale
    # the same gate as the whole-matrix comparisons at N <= 960
    assert err < 1e-11, err


def test_mixed_matrix_columns_match_oracle(setup):
    G, cols, Mo = setup
    M = G.AssembleBEMMatrix(W, precision="mixed")
    Mc = device_columns(M, cols).astype(np.complex128)
    del M
    scale = np.abs(Mo).max()
    # complex64 storage: each component rounded once (2^-24 = 6e-8 of its
    # own size); the float-float far field and the complex64 stamping add a
    # few units in the last place (measured: 1.6e-7 of the entry at worst over
    # entries above 1e-4 of the largest)
    err = np.abs(Mc - Mo)
    assert err.max() / scale < 1e-7, err.max() / scale
    big = np.abs(Mo) > 1e-4 * scale
    rel = (err[big] / np.abs(Mo[big])).max()
    assert rel < 3e-7, rel
