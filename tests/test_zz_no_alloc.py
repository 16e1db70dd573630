"""gbem_lu_solve_noalloc (static device scratch, no allocation) against
gbem_lu_solve, through the C ABI.  Kept in its own file, collected last, so it
runs both after the other GPU tests and alone in a fresh process.

The entry point serves callers that cannot allocate GPU memory at solve time
(HBM taken by their matrices, or held by another allocator's pool); besides
the results, the tests check that a call leaves both the device's free memory
and the default stream-ordered pool's usage untouched."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# cudaMemPoolAttr values (driver_types.h)
_POOL_USED_CURRENT, _POOL_USED_HIGH = 7, 8


def _cudart():
    """The CUDA runtime the library itself loaded (found through the process
    maps, so it is the same copy and the same context)."""
    import gbem
    gbem.lib()
    with open("/proc/self/maps") as f:
        paths = {ln.split()[-1] for ln in f if "libcudart.so" in ln}
    assert paths, "libcudart is not loaded"
    rt = ctypes.CDLL(sorted(paths)[0])
    rt.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    rt.cudaDeviceGetDefaultMemPool.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    rt.cudaMemPoolGetAttribute.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    rt.cudaMemPoolSetAttribute.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return rt


class _AllocWatch:
    """Free device memory and the default pool's peak usage around a call."""

    def __init__(self, device=0):
        self.rt = _cudart()
        self.pool = ctypes.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(ctypes.byref(self.pool), device) == 0

    def _pool(self, attr):
        v = ctypes.c_uint64()
        assert self.rt.cudaMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def _free(self):
        f, t = ctypes.c_size_t(), ctypes.c_size_t()
        assert self.rt.cudaMemGetInfo(ctypes.byref(f), ctypes.byref(t)) == 0
        return f.value

    def __enter__(self):
        zero = ctypes.c_uint64(0)
        assert self.rt.cudaMemPoolSetAttribute(self.pool, _POOL_USED_HIGH, ctypes.byref(zero)) == 0
        self.used0 = self._pool(_POOL_USED_CURRENT)
        self.free0 = self._free()
        return self

    def __exit__(self, *exc):
        self.free1 = self._free()
        self.used_high = self._pool(_POOL_USED_HIGH)
        return False


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
@pytest.mark.parametrize("trans", ["N", "T", "C"])
def test_noalloc_solve_matches_lu_solve(precision, tol, trans):
    from gbem._lib import lib
    L = lib()
    G, M = _factored(2, precision)  # N = 960
    rng = np.random.default_rng(7)
    B = rng.standard_normal((M.N, 11)) + 1j * rng.standard_normal((M.N, 11))  # two chunks of <= 8 columns
    X_ref = _solve(L.gbem_lu_solve, M, trans, B)
    # two calls in a row share the scratch array; both must agree with gbem_lu_solve
    watch = _AllocWatch()
    for call in range(2):
        if call == 1:
            # the second call (its kernels already loaded) must not touch the
            # device's free memory nor draw on the stream-ordered pool
            with watch:
                X = _solve(L.gbem_lu_solve_noalloc, M, trans, B)
            assert watch.free1 == watch.free0, (watch.free0, watch.free1)
            assert watch.used_high <= watch.used0, (watch.used0, watch.used_high)
        else:
            X = _solve(L.gbem_lu_solve_noalloc, M, trans, B)
        err = np.linalg.norm(X - X_ref) / np.linalg.norm(X_ref)
        assert err <= tol, err
    # and the solution solves the system it factored
    A = G.AssembleBEMMatrix(2.0, precision=precision).numpy().astype(np.complex128)
    opA = {"N": A, "T": A.T, "C": A.conj().T}[trans]
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


def test_noalloc_rejects_real_factor():
    """A real (F64) factor, the imaginary-frequency storage, is refused with
    its reason; gbem_lu_solve solves it."""
    from gbem import GbemError, RWGGeometry, mesh
    from gbem._lib import F64, check, lib
    from gbem.api import HMatrix
    V, P = mesh.icosphere(1)
    G = RWGGeometry([{"V": V, "P": P}])  # PEC sphere, N = 120
    A = G.AssembleBEMMatrixBlock(0, 0, 0.7j, real=True)
    M = HMatrix(G, F64)
    M.set(A)
    assert M.LUFactorize() == 0
    B = np.ones((M.N, 2), dtype=np.float64, order="F")
    with pytest.raises(GbemError) as e:
        check(lib().gbem_lu_solve_noalloc(M._h, b"N", 2, B.ctypes.data, M.N))
    assert "EINVAL" in str(e.value) and "complex" in str(e.value) and "gbem_lu_solve" in str(e.value)
    X = M.LUSolve(B)
    assert np.linalg.norm(A @ X - B) / np.linalg.norm(B) < 1e-12
