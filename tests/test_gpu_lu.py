"""Dense LU factor/solve on the GPU against LAPACK (numpy/scipy)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lu_host(A):
    from gbem._lib import check, lib
    import ctypes
    N = A.shape[0]
    LU = np.asfortranarray(A.astype(np.complex128))
    ipiv = np.zeros(N, dtype=np.int32)
    info = ctypes.c_int()
    st = lib().gbem_lu_factor_host(LU.ctypes.data, N, N, ipiv.ctypes.data, ctypes.byref(info))
    return st, LU, ipiv, info.value


def _solve_host(LU, ipiv, B, trans="N"):
    from gbem._lib import check, lib
    N = LU.shape[0]
    X = np.asfortranarray(B.astype(np.complex128).reshape(N, -1))
    check(lib().gbem_lu_solve_host(LU.ctypes.data, N, N, ipiv.ctypes.data, trans.encode(), X.shape[1],
                                   X.ctypes.data, N))
    return X


@pytest.mark.parametrize("N", [1, 7, 64, 257, 1000, 2049])
def test_lu_matches_lapack(N):
    import scipy.linalg as sl
    rng = np.random.default_rng(N)
    A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    st, LU, ipiv, info = _lu_host(A)
    assert st == 0 and info == 0
    lu_ref, piv_ref = sl.lu_factor(A)
    # same pivoting rule as zgetrf (|Re|+|Im|, first maximum): identical pivots
    assert np.array_equal(ipiv - 1, piv_ref)
    assert np.abs(LU - lu_ref).max() / np.abs(lu_ref).max() < 1e-11
    B = rng.standard_normal((N, 3)) + 1j * rng.standard_normal((N, 3))
    X = _solve_host(LU, ipiv, B)
    assert np.abs(A @ X - B).max() / np.abs(B).max() < 1e-9
    XT = _solve_host(LU, ipiv, B, "T")
    assert np.abs(A.T @ XT - B).max() / np.abs(B).max() < 1e-9
    XC = _solve_host(LU, ipiv, B, "C")  # zgetrs Trans = 'C': A^H x = b
    assert np.abs(A.conj().T @ XC - B).max() / np.abs(B).max() < 1e-9


def test_singular_info():
    N = 50
    rng = np.random.default_rng(1)
    A = rng.standard_normal((N, N)) + 0j
    A[:, 10] = 0.0
    st, LU, ipiv, info = _lu_host(A)
    from gbem._lib import GBEM_ESINGULAR
    assert st == GBEM_ESINGULAR and info == 11


def test_bem_matrix_c64_and_c128(golden):
    import scipy.linalg as sl
    from gbem import C64, RWGGeometry
    from helpers import fixture_surfaces, omega_of
    d = golden("ref_diel_s1_w2.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    M = G.AssembleBEMMatrix(omega_of(d))
    A = M.numpy()
    assert M.LUFactorize() == 0
    b = d["rhs0"]
    x = M.LUSolve(b)
    xr = sl.solve(A, b)
    assert np.abs(x - xr).max() / np.abs(xr).max() < 1e-10
    # the reference's own solution of its own matrix (same mesh, frequency)
    assert np.abs(x - d["kn0"]).max() / np.abs(d["kn0"]).max() < 1e-5
    M32 = G.AssembleBEMMatrix(omega_of(d), precision="mixed")
    assert M32.LUFactorize() == 0
    x32 = M32.LUSolve(b.astype(np.complex64))
    assert np.abs(x32 - xr).max() / np.abs(xr).max() < 1e-3


def test_complex64_lu_tensor_core_update():
    """C64 LU (split-BF16 tensor-core trailing updates) on a matrix large
    enough for several panels; compared with LAPACK in FP64."""
    import scipy.linalg as sl
    from gbem import C64, RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(2)
    G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}])
    M = G.AssembleBEMMatrix(2.0, precision="mixed")     # N = 960: 4 panels of 256
    A = M.numpy().astype(np.complex128)
    assert M.LUFactorize() == 0
    lu_ref, piv_ref = sl.lu_factor(A)
    # backward error of P A = L U (FP32 rounding may reorder near-tied
    # pivots, so the pivots themselves are not compared with LAPACK's)
    N = A.shape[0]
    LU = M.numpy().astype(np.complex128)
    perm = np.arange(N)
    for i, p in enumerate(M.ipiv - 1):
        perm[[i, p]] = perm[[p, i]]
    be = np.linalg.norm(A[perm] - (np.tril(LU, -1) + np.eye(N)) @ np.triu(LU)) / np.linalg.norm(A)
    assert be < 2e-4
    rng = np.random.default_rng(3)
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    x = M.LUSolve(b.astype(np.complex64)).astype(np.complex128)
    xr = sl.lu_solve((lu_ref, piv_ref), b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 2e-4


@pytest.mark.parametrize("subdiv,pec,tol", [(1, False, 1e-4), (2, False, 2e-3), (3, True, 2e-3)])
def test_complex64_lu_random_matrix(subdiv, pec, tol):
    """C64 LU of a random matrix uploaded into a BEM-sized HMatrix.  N = 240
    is one panel (recursive cluster leaves; split-BF16 tensor-core updates at
    the upper recursion levels); N = 960, 1920 add split-BF16 trailing
    updates.  The split keeps about 16 mantissa bits per product."""
    import scipy.linalg as sl
    from gbem import C64, RWGGeometry, mesh
    from gbem.api import HMatrix, Material
    V, P = mesh.icosphere(subdiv)
    G = RWGGeometry([{"V": V, "P": P, "material": None if pec else Material(2.25)}])
    M = HMatrix(G, C64)
    N = M.N
    rng = np.random.default_rng(N)
    A = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    M.set(A)
    assert M.LUFactorize() == 0
    A = A.astype(np.complex128)
    LU = M.numpy().astype(np.complex128)
    L = np.tril(LU, -1) + np.eye(N)
    U = np.triu(LU)
    perm = np.arange(N)
    for i, p in enumerate(M.ipiv - 1):  # LAPACK-style sequential interchanges
        assert i <= p < N
        perm[[i, p]] = perm[[p, i]]
    # backward error of P A = L U; the |Re|+|Im| pivot bounds |l| by sqrt(2)
    assert np.linalg.norm(A[perm] - L @ U) / np.linalg.norm(A) < tol
    assert np.abs(L).max() <= np.sqrt(2.0) * (1 + 1e-5)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    x = M.LUSolve(b.astype(np.complex64)).astype(np.complex128)
    xr = sl.solve(A, b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 500 * tol



def test_panel_width_tuning_is_reported():
    """The complex-FP32 LU picks its panel width per 1024-row bucket of N by
    timing both widths on a scratch copy of the bucket's first matrix; the
    choice is reported by gbem_lu_tuning and the factorisation that used it
    solves the system."""
    from gbem import C64, RWGGeometry, mesh
    from gbem.api import HMatrix, LUTuning, Material
    V, P = mesh.icosphere(2)
    G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25)}])
    M = HMatrix(G, C64)
    N = M.N  # 1920
    rng = np.random.default_rng(7)
    A = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    M.set(A)
    assert M.LUFactorize() == 0
    t = LUTuning(0)
    print("LU tuning:", t)
    assert t["panel_width_by_N"].get("1024-2047") in (128, 256)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    x = M.LUSolve(b.astype(np.complex64)).astype(np.complex128)
    A = A.astype(np.complex128)
    # normwise backward error of the complex-FP32 solve (split-BF16 updates
    # keep ~16 bits per product: 1.0e-4 measured at this size)
    assert np.linalg.norm(A @ x - b) / (np.linalg.norm(A, 2) * np.linalg.norm(x)) < 1e-3
