"""Packed symmetric storage (HMatrix's LHM_SYMMETRIC) on the GPU against
LAPACK's own dsptrf/zsptrf and dsptrs/zsptrs (UPLO = 'U'), the routines
HMatrix::LUFactorize/LUSolve call for it (LBWrappers.cc:159-166, 175-236):
random real and complex symmetric matrices (1 x 1 and 2 x 2 pivots), a
matrix with a zero column, and the packed T block of a PEC sphere at
imaginary frequency (scuff-cas3D's storage, CreateSC3Data.cc:110) and of a
dielectric sphere at real frequency."""
import numpy as np
import pytest

from helpers import lapack_sp, pack_upper, unpack_upper

pytestmark = pytest.mark.gpu


def _check(AP, n, B, ftol=1e-12, xtol=1e-10):
    from gbem.api import SymmetricLUFactorize, SymmetricLUSolve
    Fl, pl, il, Xl = lapack_sp(AP, n, B)
    F = np.array(AP, copy=True)
    ipiv, info = SymmetricLUFactorize(F, n)
    assert info == il
    # same pivots as LAPACK (ties are measure-zero on these inputs)
    assert np.array_equal(ipiv, pl)
    assert np.abs(F - Fl).max() <= ftol * max(1.0, np.abs(Fl).max())
    X = SymmetricLUSolve(F, n, ipiv, B)
    assert np.abs(X - Xl).max() <= xtol * np.abs(Xl).max()
    return ipiv, X


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("n", [1, 2, 97, 640])
def test_random_symmetric_matches_lapack(dt, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if dt is np.complex128 else 0)
    A = (A + A.T).astype(dt)
    # small diagonal: Bunch-Kaufman takes 2 x 2 pivots and interchanges
    A[np.diag_indices(n)] *= 0.05
    B = rng.standard_normal((n, 5)).astype(dt)
    ipiv, X = _check(pack_upper(A), n, B)
    if n > 2:
        assert (ipiv < 0).any() and (np.abs(ipiv) != np.arange(1, n + 1)).any()
    assert np.abs(A @ X - B).max() <= 1e-9 * np.abs(A).max() * np.abs(X).max()


def test_zero_column_sets_info_like_lapack():
    rng = np.random.default_rng(9)
    n = 40
    A = rng.standard_normal((n, n))
    A = A + A.T
    A[:, 17] = 0.0
    A[17, :] = 0.0
    from gbem.api import SymmetricLUFactorize
    Fl, pl, il = lapack_sp(pack_upper(A), n)
    F = pack_upper(A)
    ipiv, info = SymmetricLUFactorize(F, n)
    assert il > 0 and info == il
    assert np.array_equal(ipiv, pl)


@pytest.mark.parametrize("case", ["pec_xi", "diel_w"])
def test_packed_t_block_assembles_and_factors(case):
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(2)
    if case == "pec_xi":
        G = RWGGeometry([{"V": V, "P": P}])  # N = 480
        w, real = 0.9j, True
    else:
        G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}])  # N = 960, complex symmetric
        w, real = 2.0, False
    n = G.NumBFs(0)
    AP = G.AssembleBEMMatrixBlockPacked(0, w, real=real)
    full = G.AssembleBEMMatrixBlock(0, 0, w, real=real)
    assert np.array_equal(unpack_upper(AP, n), np.triu(full))
    assert np.array_equal(full, full.T)
    rng = np.random.default_rng(2)
    B = rng.standard_normal((n, 3)).astype(AP.dtype)
    ipiv, X = _check(AP, n, B)
    assert np.abs(full @ X - B).max() <= 1e-9 * np.abs(B).max()
