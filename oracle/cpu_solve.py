"""The CPU reference solve, in bounded slices (TEST INFRASTRUCTURE ONLY: the
CPU baseline of bench.py, never the product).

One solve of the reference's path on the host cores, at full size, as the
reference performs it (scuff-scatter: AssembleBEMMatrix, LUFactorize, LUSolve;
scuff-scatter.cc:402-495):

* assembly: the oracle's restatement of AssembleBEMMatrix (OpenMP over edge
  pairs of the upper triangle, gbem_oracle.c), warm -- the static near-pair
  integrals memoised beforehand, as the reference's FIPPI cache holds them
  after the first frequency (FIPPICache.cc:135-187);
* factorisation: LAPACK's blocked right-looking LU (the algorithm of zgetrf:
  per panel, zgetrf on the panel, zlaswp on both sides, ztrsm for U12, zgemm
  for the trailing matrix), in OpenBLAS from scipy, on all host threads;
* solve: zgetrs with the right-hand sides (LBWrappers.cc:208-236).

SlicedSolve cuts that work into parts run one after another: a column stripe
of the assembly holding a known fraction of the upper triangle's edge pairs,
or a run of LU panel steps holding a known fraction of its flops.  Each part
is real work on the full-size matrices, so a caller can time some parts and
know what fraction of one solve it timed.  The LU runs on a seeded random
matrix of the same size, whose LU costs what the BEM matrix's does (partial
pivoting swaps rows either way; the arithmetic does not depend on the
values); the assembly writes the BEM matrix itself.
"""
from __future__ import annotations

import ctypes
import glob
import os
import platform
import time

import numpy as np

from . import oracle


def _openblas():
    """(ctypes library, symbol prefix) of the OpenBLAS scipy.linalg uses."""
    import scipy.linalg  # noqa: F401  (loads its OpenBLAS)
    with open("/proc/self/maps") as f:
        paths = sorted({ln.split()[-1] for ln in f if "openblas" in ln.lower() and ".so" in ln})
    if not paths:
        import scipy
        d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
        paths = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    for p in paths:
        L = ctypes.CDLL(p)
        for pre in ("scipy_", ""):
            if hasattr(L, pre + "zgemm_") and hasattr(L, pre + "zgetrf_"):
                return L, pre
    raise RuntimeError("no OpenBLAS with zgemm_/zgetrf_ found")


def cpu_model():
    """The host CPU as /proc/cpuinfo names it (model name, or the Arm
    implementer/part pair), with the machine type."""
    name = None
    try:
        info = open("/proc/cpuinfo").read()
        for key in ("model name", "Model", "cpu model"):
            for ln in info.splitlines():
                if ln.lower().startswith(key.lower()) and ":" in ln:
                    name = ln.split(":", 1)[1].strip()
                    break
            if name:
                break
        if not name:
            imp = [ln.split(":")[1].strip() for ln in info.splitlines() if ln.startswith("CPU implementer")]
            part = [ln.split(":")[1].strip() for ln in info.splitlines() if ln.startswith("CPU part")]
            if imp and part:
                name = "arm implementer %s part %s" % (imp[0], part[0])
    except OSError:
        pass
    return "%s (%s)" % (name or "unknown", platform.machine())


class BlockedLU:
    """zgetrf's blocked right-looking algorithm on a column-major complex128
    N x N array, one panel at a time, through LAPACK/BLAS calls on the array
    in place (1-based pivots in ipiv, as zgetrf returns them)."""

    def __init__(self, A, nb=256):
        assert A.dtype == np.complex128 and A.flags.f_contiguous and A.shape[0] == A.shape[1]
        self.A, self.N, self.nb = A, A.shape[0], nb
        self.ipiv = np.zeros(self.N, dtype=np.int32)
        self.L, pre = _openblas()
        self.f = {n: getattr(self.L, pre + n + "_") for n in ("zgetrf", "zlaswp", "ztrsm", "zgemm", "zgetrs")}
        self.npanels = (self.N + nb - 1) // nb
        self.info = 0

    def panel_flops(self, k):
        """Algorithmic flops of panel step k: complex flops, 4x the real
        counts of the panel LU (m w^2 - w^3/3) and of the triangular solve
        (w^2 r), and 8 r^2 w for the trailing update."""
        N, nb = self.N, self.nb
        j = k * nb
        w = min(nb, N - j)
        m = N - j
        r = N - j - w
        return 4.0 * (m * w * w - w ** 3 / 3.0) + 4.0 * r * w * w + 8.0 * r * r * w

    def total_flops(self):
        return sum(self.panel_flops(k) for k in range(self.npanels))

    def _p(self, i, j):
        return ctypes.c_void_p(self.A.ctypes.data + 16 * (i + j * self.N))

    def panels(self, k0, k1):
        """Factor panel steps [k0, k1) (must follow steps [0, k0))."""
        c_int = ctypes.c_int
        N, nb = self.N, self.nb
        one = np.array([1.0, 0.0])
        mone = np.array([-1.0, 0.0])
        ld = c_int(N)
        for k in range(k0, min(k1, self.npanels)):
            j = k * nb
            w = min(nb, N - j)
            m = N - j
            info = c_int(0)
            piv = np.zeros(w, dtype=np.int32)
            self.f["zgetrf"](ctypes.byref(c_int(m)), ctypes.byref(c_int(w)), self._p(j, j), ctypes.byref(ld),
                             piv.ctypes.data_as(ctypes.c_void_p), ctypes.byref(info))
            if info.value > 0 and self.info == 0:
                self.info = info.value + j
            self.ipiv[j:j + w] = piv + j
            # interchanges on the columns left and right of the panel
            k1_, k2_, inc = c_int(j + 1), c_int(j + w), c_int(1)
            if j > 0:
                self.f["zlaswp"](ctypes.byref(c_int(j)), self._p(0, 0), ctypes.byref(ld), ctypes.byref(k1_),
                                 ctypes.byref(k2_), self.ipiv.ctypes.data_as(ctypes.c_void_p), ctypes.byref(inc))
            r = N - j - w
            if r > 0:
                self.f["zlaswp"](ctypes.byref(c_int(r)), self._p(0, j + w), ctypes.byref(ld), ctypes.byref(k1_),
                                 ctypes.byref(k2_), self.ipiv.ctypes.data_as(ctypes.c_void_p), ctypes.byref(inc))
                self.f["ztrsm"](b"L", b"L", b"N", b"U", ctypes.byref(c_int(w)), ctypes.byref(c_int(r)),
                                one.ctypes.data_as(ctypes.c_void_p), self._p(j, j), ctypes.byref(ld),
                                self._p(j, j + w), ctypes.byref(ld))
                self.f["zgemm"](b"N", b"N", ctypes.byref(c_int(r)), ctypes.byref(c_int(r)), ctypes.byref(c_int(w)),
                                mone.ctypes.data_as(ctypes.c_void_p), self._p(j + w, j), ctypes.byref(ld),
                                self._p(j, j + w), ctypes.byref(ld), one.ctypes.data_as(ctypes.c_void_p),
                                self._p(j + w, j + w), ctypes.byref(ld))

    def solve(self, B):
        """zgetrs 'N' on B (N x nrhs, column-major complex128) in place."""
        c_int = ctypes.c_int
        assert B.dtype == np.complex128 and B.flags.f_contiguous
        info = c_int(0)
        self.f["zgetrs"](b"N", ctypes.byref(c_int(self.N)), ctypes.byref(c_int(B.shape[1])),
                         self._p(0, 0), ctypes.byref(c_int(self.N)), self.ipiv.ctypes.data_as(ctypes.c_void_p),
                         B.ctypes.data_as(ctypes.c_void_p), ctypes.byref(c_int(self.N)), ctypes.byref(info))
        return info.value


class SlicedSolve:
    """One full-size CPU solve of a dielectric sphere (icosphere ``subdiv``,
    PMCHWT, eps at omega), cut into slices."""

    def __init__(self, subdiv=4, eps=2.25 + 0.01j, omega=2.0, nrhs=4, seed=0, nb=256, warm=True):
        from gbem import mesh
        V, P = mesh.icosphere(subdiv)
        self.S = oracle.Surface(V, P)
        self.ne = self.S.edges()[0].shape[0]
        self.N = 2 * self.ne
        self.eps, self.omega, self.nrhs = [1.0, eps], omega, nrhs
        t0 = time.perf_counter()
        self.near_pairs = oracle.warm_near(self.S) if warm else 0
        self.t_warm = time.perf_counter() - t0
        self.M = np.zeros((self.N, self.N), dtype=np.complex128, order="F")
        rng = np.random.default_rng(seed)
        A = np.empty((self.N, self.N), dtype=np.complex128, order="F")
        for c0 in range(0, self.N, 1024):  # column blocks keep the temporaries small
            c1 = min(self.N, c0 + 1024)
            A[:, c0:c1] = rng.standard_normal((self.N, c1 - c0)) + 1j * rng.standard_normal((self.N, c1 - c0))
        self.lu = BlockedLU(A, nb)
        self.B = np.asfortranarray(rng.standard_normal((self.N, nrhs)) + 1j * rng.standard_normal((self.N, nrhs)))
        self.pairs_total = self.ne * (self.ne + 1) // 2

    def stripe_bounds(self, S):
        """Column-edge boundaries of S stripes with equal edge-pair counts
        (column edge eb holds eb + 1 pairs of the upper triangle)."""
        b = [0]
        for j in range(1, S):
            b.append(int(round(self.ne * np.sqrt(j / S))))
        b.append(self.ne)
        return b

    def assemble(self, eb0, eb1):
        """Assemble column edges [eb0, eb1); returns (seconds, pair fraction)."""
        t0 = time.perf_counter()
        oracle.assemble_stripe(self.S, False, self.omega, self.eps, [1.0, 1.0], eb0, eb1, self.M)
        dt = time.perf_counter() - t0
        pairs = (eb1 * (eb1 + 1) - eb0 * (eb0 + 1)) // 2
        return dt, pairs / self.pairs_total

    def panel_bounds(self, S):
        """Panel-step boundaries of S runs with about equal flops (runs may
        be empty when S exceeds the number of panels)."""
        fl = np.cumsum([self.lu.panel_flops(k) for k in range(self.lu.npanels)])
        b = [0]
        for j in range(1, S):
            b.append(min(int(np.searchsorted(fl, fl[-1] * j / S)) + 1, self.lu.npanels))
        b.append(self.lu.npanels)
        return b

    def factor(self, k0, k1):
        """Panel steps [k0, k1); returns (seconds, flop fraction)."""
        t0 = time.perf_counter()
        self.lu.panels(k0, k1)
        dt = time.perf_counter() - t0
        fl = sum(self.lu.panel_flops(k) for k in range(k0, min(k1, self.lu.npanels)))
        return dt, fl / self.lu.total_flops()

    def solve(self):
        t0 = time.perf_counter()
        X = self.B.copy(order="F")
        self.lu.solve(X)
        return time.perf_counter() - t0
