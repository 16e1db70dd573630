"""gbem_lu_solve_noalloc (static device scratch, no allocation) against
gbem_lu_solve, through the C ABI.  Kept in its own file, collected last, so it
runs both after the other GPU tests and alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(fn, M, trans, B):
    from gbem._lib import check
    X = np.array(B, dtype=M.np_dtype, order="F", copy=True)
    check(fn(M._h, trans.encode(), X.shape[1], X.ctypes.data, M.N))
    return X


def _factored(subdiv, precision):
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(subdiv)
    G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}])
    M = G.AssembleBEMMatrix(2.0, precision=precision)
    assert M.LUFactorize() == 0
    return G, M


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_noalloc_solve_matches_lu_solve(precision, tol, trans):
    from gbem._lib import lib
    L = lib()
    G, M = _factored(2, precision)  # N = 960
    rng = np.random.default_rng(7)
    B = rng.standard_normal((M.N, 11)) + 1j * rng.standard_normal((M.N, 11))  # two chunks of <= 8 columns
    X_ref = _solve(L.gbem_lu_solve, M, trans, B)
    # two calls in a row share the scratch array; both must agree with gbem_lu_solve
    for _ in range(2):
        X = _solve(L.gbem_lu_solve_noalloc, M, trans, B)
        err = np.linalg.norm(X - X_ref) / np.linalg.norm(X_ref)
        assert err <= tol, err
    # and the solution solves the system it factored
    A = G.AssembleBEMMatrix(2.0, precision=precision).numpy().astype(np.complex128)
    opA = A if trans == "N" else A.T
    res = np.linalg.norm(opA @ X.astype(np.complex128) - B) / np.linalg.norm(B)
    assert res <= (1e-10 if precision == "fp64" else 1e-4), res


def test_noalloc_rejects_n_beyond_scratch():
    from gbem import GbemError, RWGGeometry, mesh
    from gbem._lib import C128, check, lib
    from gbem.api import HMatrix, Material
    V, P = mesh.icosphere(4)  # dielectric: N = 15360 > 13088
    G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25)}])
    M = HMatrix(G, C128)
    B = np.zeros((M.N, 1), dtype=np.complex128, order="F")
    with pytest.raises(GbemError) as e:
        check(lib().gbem_lu_solve_noalloc(M._h, b"N", 1, B.ctypes.data, M.N))
    assert "EINVAL" in str(e.value) and "13088" in str(e.value)
