"""Shared helpers for the tests: build gbem / oracle geometries from fixtures."""
import numpy as np


def fixture_surfaces(d):
    """(list of gbem surface dicts, oracle args) from a ref_*.npz fixture."""
    from gbem.api import Material
    n = int(d["objects"])
    gs, regs, pec, eps, mu = [], [], [], [1.0], [1.0]
    for i in range(n):
        V = d["V%d" % i] + d["disp%d" % i]
        P = d["P%d" % i]
        mat = str(d["mat%d" % i])
        if mat == "PEC":
            gs.append({"V": V, "P": P, "material": None})
            regs.append((0, -1)); pec.append(True)
        else:
            m = Material.parse(mat)
            gs.append({"V": V, "P": P, "material": m})
            eps.append(m.eps); mu.append(m.mu)
            regs.append((0, len(eps) - 1)); pec.append(False)
    return gs, (regs, pec, eps, mu)


def omega_of(d):
    return d["omega"][0] + 1j * d["omega"][1]


def relerr(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def cudart():
    """The CUDA runtime the library loaded (found through the process maps,
    so calls share its context)."""
    import ctypes
    import gbem
    gbem.lib()
    with open("/proc/self/maps") as f:
        paths = {ln.split()[-1] for ln in f if "libcudart.so" in ln}
    assert paths, "libcudart is not loaded"
    rt = ctypes.CDLL(sorted(paths)[0])
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return rt


def device_columns(M, cols):
    """Columns ``cols`` of a device-resident HMatrix, copied to the host
    without downloading the whole matrix."""
    import ctypes
    rt = cudart()
    p, ld = M.device_ptr()
    es = np.dtype(M.np_dtype).itemsize
    out = np.zeros((M.N, len(cols)), dtype=M.np_dtype, order="F")
    for j, c in enumerate(cols):
        src = p + int(c) * ld * es
        dst = out.ctypes.data + j * M.N * es
        assert rt.cudaMemcpy(ctypes.c_void_p(dst), ctypes.c_void_p(src), M.N * es, 2) == 0  # DeviceToHost
    return out


def lapack_sp(AP, N, B=None):
    """LAPACK's own dsptrf/zsptrf and dsptrs/zsptrs ('U') from the OpenBLAS
    scipy ships (the routines HMatrix::LUFactorize/LUSolve call for packed
    symmetric storage): returns (factor, ipiv, info[, X])."""
    import ctypes
    from oracle.cpu_solve import _openblas
    L, pre = _openblas()
    t = "z" if np.iscomplexobj(AP) else "d"
    F = np.array(AP, copy=True)
    ipiv = np.zeros(N, dtype=np.int32)
    info = ctypes.c_int(0)
    n = ctypes.c_int(N)
    getattr(L, pre + t + "sptrf_")(b"U", ctypes.byref(n), F.ctypes.data_as(ctypes.c_void_p),
                                   ipiv.ctypes.data_as(ctypes.c_void_p), ctypes.byref(info))
    if B is None:
        return F, ipiv, info.value
    X = np.array(B, dtype=F.dtype, order="F", copy=True).reshape(N, -1, order="F")
    info2 = ctypes.c_int(0)
    getattr(L, pre + t + "sptrs_")(b"U", ctypes.byref(n), ctypes.byref(ctypes.c_int(X.shape[1])),
                                   F.ctypes.data_as(ctypes.c_void_p), ipiv.ctypes.data_as(ctypes.c_void_p),
                                   X.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n), ctypes.byref(info2))
    return F, ipiv, info.value, X


def pack_upper(A):
    """HMatrix's LHM_SYMMETRIC packing of a square array's upper triangle."""
    n = A.shape[0]
    return np.concatenate([A[:j + 1, j] for j in range(n)])


def unpack_upper(AP, n):
    A = np.zeros((n, n), dtype=AP.dtype)
    o = 0
    for j in range(n):
        A[:j + 1, j] = AP[o:o + j + 1]
        o += j + 1
    return A
