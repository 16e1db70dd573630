"""ctypes wrapper of the CPU oracle (oracle/gbem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg as the checker.  The product never calls it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gbem_oracle.c")
LIB = os.path.join(HERE, "_build", "liboracle.so")
REFDUMP = os.path.join(HERE, "_ref", "refdump")

ALG_NAMES = {0: "LO", 1: "HO", 2: "TD", 3: "HKTD", 4: "DESING"}


def build():
    """Compile the oracle (gcc, OpenMP)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-w", "-ffp-contract=off", "-o", tmp, SRC, "-lm"],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


def reference_tree():
    """The reference source tree, if this machine has one: the directory named
    by SCUFF_REF, else a checkout named ``reference`` beside this repository.
    None where neither exists (the GPU host has no reference tree and uses the
    committed fixtures)."""
    cands = [os.environ.get("SCUFF_REF"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "libs", "libscuff")):
            return os.path.abspath(c)
    return None


def build_reference(ref=None, jobs=8):
    """Build the reference from its sources into oracle/_ref (only where the
    reference tree exists; the GPU host uses the committed fixtures)."""
    ref = ref or reference_tree()
    if not ref or not os.path.isdir(ref):
        return None
    subprocess.run(["make", "-C", os.path.join(HERE, "ref"), "REF=" + ref, "-j%d" % jobs], check=True,
                   capture_output=True)
    return REFDUMP


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.ora_surface_new.restype = P
        L.ora_surface_new.argtypes = [I, P, I, P]
        L.ora_surface_free.argtypes = [P]
        L.ora_surface_num_edges.argtypes = [P]
        L.ora_surface_edges.argtypes = [P, P, P]
        L.ora_ppi_c.argtypes = [P, I, I, I, I, D, D, P, P]
        L.ora_qifippi_c.argtypes = [P, I, I, I, P, P]
        L.ora_set_orders.argtypes = [I, I, I, I, I]
        L.ora_assemble.argtypes = [I, P, P, P, D, D, P, P, P, I]
        L.ora_gc_matrix.argtypes = [P, D, D, P, P]
        L.ora_assemble_cols.argtypes = [I, P, P, P, D, D, P, P, I, P, P, I]
        L.ora_assemble_stripe.argtypes = [P, I, I, I, D, D, P, P, I, I, P, I]
        L.ora_warm_near.argtypes = [P]
        L.ora_warm_near.restype = ctypes.c_longlong
        _lib = L
    return _lib


class Surface:
    def __init__(self, V, P):
        self.V = np.ascontiguousarray(V, dtype=np.float64)
        self.P = np.ascontiguousarray(P, dtype=np.int32)
        self.h = lib().ora_surface_new(len(self.V), self.V.ctypes.data, len(self.P), self.P.ctypes.data)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_surface_free(self.h)
            self.h = None

    def edges(self):
        n = lib().ora_surface_num_edges(self.h)
        E = np.zeros((n, 8), dtype=np.int32)
        L = np.zeros(n)
        lib().ora_surface_edges(self.h, E.ctypes.data, L.ctypes.data)
        return E, L

    def ppi(self, pa, iqa, pb, iqb, k):
        k = complex(k)
        H = np.zeros(4)
        ncv = ctypes.c_int()
        alg = lib().ora_ppi_c(self.h, pa, iqa, pb, iqb, k.real, k.imag, H.ctypes.data, ctypes.byref(ncv))
        return np.array([H[0] + 1j * H[1], H[2] + 1j * H[3]]), alg, ncv.value

    def qifippi(self, pa, pb, n=24):
        out = np.zeros(33)
        order = np.zeros(6, dtype=np.int32)
        ncv = lib().ora_qifippi_c(self.h, pa, pb, n, out.ctypes.data, order.ctypes.data)
        return out, ncv, order


def gc_matrices(surface, k):
    """GC[0], GC[1] of every edge pair of one surface at wavenumber k
    (EdgeEdgeInteractions.cc:183-188), as two ne x ne complex arrays."""
    k = complex(k)
    ne = lib().ora_surface_num_edges(surface.h)
    g0 = np.zeros((ne, ne), dtype=np.complex128, order="F")
    g1 = np.zeros((ne, ne), dtype=np.complex128, order="F")
    lib().ora_gc_matrix(surface.h, k.real, k.imag, g0.ctypes.data, g1.ctypes.data)
    return g0, g1


ZVAC = 376.73031346177


def emt_pscat(surface, pec, omega, KN, eps0=1.0, mu0=1.0):
    """EMT scattered power of one surface in the exterior region
    (EMTPFT.cc:642-700, self-surface branch): with QKK = mu w GC0,
    QNN = eps w GC0 and ikC = i k GC1 (GetScatteredPFTIntegrals,
    EMTPFT.cc:333-352),  P = 1/2 sum_ab [ZVAC Re(K_a* K_b) Im QKK
    + Re(N_a* N_b)/ZVAC Im QNN + Im(K_a* N_b - N_a* K_b) Im ikC],
    K and N = -ZVAC * KN[odd] as in RWGGeometry::GetKNCoefficients."""
    omega = complex(omega)
    k0 = np.sqrt(complex(eps0) * complex(mu0)) * omega
    g0, g1 = gc_matrices(surface, k0)
    KN = np.asarray(KN)
    if pec:
        K, N = KN, np.zeros_like(KN)
    else:
        K, N = KN[0::2], -ZVAC * KN[1::2]
    re = lambda a, b: np.real(np.conj(a)[:, None] * b[None, :])
    im = lambda a, b: np.imag(np.conj(a)[:, None] * b[None, :])
    p = ZVAC * np.sum(re(K, K) * np.imag(mu0 * omega * g0))
    p += np.sum(re(N, N) * np.imag(eps0 * omega * g0)) / ZVAC
    p += np.sum((im(K, N) - im(N, K)) * np.imag(1j * k0 * g1))
    return 0.5 * p


def assemble(surfaces, regions, pec, omega, eps, mu):
    """Full BEM matrix of a compact geometry (complex128, N x N).

    surfaces: list of Surface; regions: list of (exterior, interior) region
    indices; pec: list of bools; eps/mu: complex per region."""
    N = sum(s.edges()[0].shape[0] * (1 if p else 2) for s, p in zip(surfaces, pec))
    handles = (ctypes.c_void_p * len(surfaces))(*[s.h for s in surfaces])
    reg = np.array([r for pair in regions for r in pair], dtype=np.int32)
    pe = np.array([1 if p else 0 for p in pec], dtype=np.int32)
    ep = np.array([[complex(e).real, complex(e).imag] for e in eps], dtype=np.float64).ravel()
    mm = np.array([[complex(m).real, complex(m).imag] for m in mu], dtype=np.float64).ravel()
    M = np.zeros((N, N), dtype=np.complex128, order="F")
    omega = complex(omega)
    lib().ora_assemble(len(surfaces), handles, reg.ctypes.data, pe.ctypes.data, omega.real, omega.imag,
                       ep.ctypes.data, mm.ctypes.data, M.ctypes.data, N)
    return M


def assemble_cols(surfaces, regions, pec, omega, eps, mu, cols):
    """Whole columns ``cols`` (every row) of the matrix ``assemble`` returns,
    equal to its columns entry for entry; for matrices too large to assemble
    whole on the CPU.  Returns an N x len(cols) complex128 array."""
    N = sum(s.edges()[0].shape[0] * (1 if p else 2) for s, p in zip(surfaces, pec))
    handles = (ctypes.c_void_p * len(surfaces))(*[s.h for s in surfaces])
    reg = np.array([r for pair in regions for r in pair], dtype=np.int32)
    pe = np.array([1 if p else 0 for p in pec], dtype=np.int32)
    ep = np.array([[complex(e).real, complex(e).imag] for e in eps], dtype=np.float64).ravel()
    mm = np.array([[complex(m).real, complex(m).imag] for m in mu], dtype=np.float64).ravel()
    cl = np.ascontiguousarray(cols, dtype=np.int32)
    if cl.size and (cl.min() < 0 or cl.max() >= N):
        raise ValueError("column index out of range")
    M = np.zeros((N, len(cl)), dtype=np.complex128, order="F")
    omega = complex(omega)
    lib().ora_assemble_cols(len(surfaces), handles, reg.ctypes.data, pe.ctypes.data, omega.real, omega.imag,
                            ep.ctypes.data, mm.ctypes.data, len(cl), cl.ctypes.data, M.ctypes.data, N)
    return M


def assemble_stripe(surface, pec, omega, eps, mu, eb0, eb1, M):
    """ora_assemble's loop over the column edges [eb0, eb1) of a
    single-surface geometry (exterior region 0, interior region 1 unless
    PEC), added into the full N x N complex128 column-major M: the upper
    triangle of those columns."""
    ep = np.array([[complex(e).real, complex(e).imag] for e in eps], dtype=np.float64).ravel()
    mm = np.array([[complex(m).real, complex(m).imag] for m in mu], dtype=np.float64).ravel()
    assert M.dtype == np.complex128 and M.flags.f_contiguous
    omega = complex(omega)
    lib().ora_assemble_stripe(surface.h, 0, -1 if pec else 1, 1 if pec else 0, omega.real, omega.imag,
                              ep.ctypes.data, mm.ctypes.data, int(eb0), int(eb1), M.ctypes.data, M.shape[0])


def warm_near(surface):
    """Compute and memoise the static near-pair integrals of every near pair
    of a surface (the warm state of the reference's FIPPI cache)."""
    return lib().ora_warm_near(surface.h)


def set_orders(td3=32, td2=20, td1=14, fip0=24, fip12=16):
    lib().ora_set_orders(td3, td2, td1, fip0, fip12)
