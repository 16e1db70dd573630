"""The packed-symmetric test helpers against numpy (no GPU): LAPACK's
dsptrf/dsptrs reached through the OpenBLAS scipy ships solve a symmetric
system, and packing round-trips."""
import numpy as np

from helpers import lapack_sp, pack_upper, unpack_upper


def test_lapack_sp_solves_and_packing_round_trips():
    rng = np.random.default_rng(3)
    for dt in (np.float64, np.complex128):
        n = 57
        A = rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if dt is np.complex128 else 0)
        A = (A + A.T).astype(dt)
        AP = pack_upper(A)
        assert np.array_equal(unpack_upper(AP, n), np.triu(A))
        B = rng.standard_normal((n, 3)).astype(dt)
        F, ipiv, info, X = lapack_sp(AP, n, B)
        assert info == 0
        assert np.abs(A @ X - B).max() < 1e-10 * np.abs(B).max() * np.abs(A).max()
