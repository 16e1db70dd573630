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
