"""Python mirror of the reference's API for the BEM hot path.

``RWGGeometry`` mirrors scuff::RWGGeometry (libs/libscuff/libscuff.h:340-634)
for what the hot path needs -- ``TotalBFs``, ``AllocateBEMMatrix``,
``AssembleBEMMatrix``, ``AssembleRHSVector`` -- and ``HMatrix`` mirrors
libhmat's HMatrix for ``LUFactorize``/``LUSolve`` (LBWrappers.cc:151-236).
Everything runs through the C ABI of libgbem.so on the GPU.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from . import _lib
from ._lib import C128, C64, F64, PREC_FP64, PREC_MIXED, check, lib
from .mesh import read_msh

ZVAC = 376.73031346177


class Material:
    """Constant (frequency-independent) eps and mu, like the reference's
    CONST_EPS_..._MU_... materials (libs/libMatProp/libMatProp.cc:205-299)."""

    def __init__(self, eps=1.0, mu=1.0):
        self.eps = complex(eps)
        self.mu = complex(mu)

    @classmethod
    def parse(cls, name):
        if name is None or name.upper() in ("PEC",):
            return None
        if name.upper() == "VACUUM":
            return cls()
        m = re.match(r"CONST_(.*)$", name, re.I)
        if not m:
            raise ValueError("only CONST_ materials are supported: %r" % name)
        toks = m.group(1).split("_")
        eps, mu = 1.0, 1.0
        for i in range(0, len(toks) - 1, 2):
            val = _parse_cval(toks[i + 1])
            if toks[i].upper() == "EPS":
                eps = val
            elif toks[i].upper() == "MU":
                mu = val
        return cls(eps, mu)


def _parse_cval(s):
    m = re.match(r"^([-+0-9.eE]+?)([-+])([0-9.eE]+)[iI]$", s)
    if m:
        re_, sg, im = m.groups()
        return complex(float(re_), (1 if sg == "+" else -1) * float(im))
    return complex(float(s), 0.0)


class HMatrix:
    """A device-resident N x N BEM matrix (complex128 or complex64)."""

    def __init__(self, geometry, dtype=C128):
        self.geometry = geometry
        self.dtype = dtype
        self.N = geometry.TotalBFs
        h = ctypes.c_void_p()
        check(lib().gbem_matrix_create(geometry._h, dtype, ctypes.byref(h)))
        self._h = h
        self.ipiv = None
        self.info = None

    def __del__(self):
        if getattr(self, "_h", None):
            lib().gbem_matrix_destroy(self._h)
            self._h = None

    @property
    def np_dtype(self):
        return {C128: np.complex128, C64: np.complex64, F64: np.float64}[self.dtype]

    def device_ptr(self):
        p, ld = ctypes.c_void_p(), ctypes.c_int()
        check(lib().gbem_matrix_device_ptr(self._h, ctypes.byref(p), ctypes.byref(ld)))
        return p.value, ld.value

    def numpy(self):
        """The matrix as a column-major numpy array (M[r, c])."""
        a = np.empty((self.N, self.N), dtype=self.np_dtype, order="F")
        check(lib().gbem_matrix_download(self._h, a.ctypes.data, self.N))
        return a

    def set(self, a):
        a = np.asfortranarray(a, dtype=self.np_dtype)
        check(lib().gbem_matrix_upload(self._h, a.ctypes.data, self.N))

    def LUFactorize(self):
        """In-place LU with partial pivoting; returns LAPACK's info (0 = ok)."""
        ipiv = np.zeros(self.N, dtype=np.int32)
        info = ctypes.c_int()
        st = lib().gbem_lu_factor(self._h, ipiv.ctypes.data, ctypes.byref(info))
        if st not in (_lib.GBEM_OK, _lib.GBEM_ESINGULAR):
            check(st)
        self.ipiv, self.info = ipiv, info.value
        return info.value

    def LogAbsDet(self):
        """log|det M| of this factored matrix: sum of log|U(n,n)| over its LU
        factor's diagonal (GetLNDetMInvMInf, CasimirIntegrand.cc:50-63)."""
        v = ctypes.c_double()
        check(lib().gbem_lu_log_abs_det(self._h, ctypes.byref(v)))
        return v.value

    def TraceMInvdM(self, dM, ncols=None):
        """Tr over the first ncols diagonal entries of M^-1 dM for this
        factored matrix and dM (an HMatrix of the same size and type, or an
        N x ncols array), the scuff-cas3D force/torque integrand
        (GetTraceMInvdM, CasimirIntegrand.cc:100-146: force = -2 Re/(2 pi))."""
        tr = np.zeros(2)
        if isinstance(dM, HMatrix):
            check(lib().gbem_lu_trace(self._h, dM._h, ncols or self.N, tr.ctypes.data))
        else:
            B = np.asfortranarray(np.asarray(dM, dtype=self.np_dtype).reshape(self.N, -1))
            check(lib().gbem_lu_trace_host(self._h, B.ctypes.data, self.N, ncols or B.shape[1], tr.ctypes.data))
        return complex(tr[0], tr[1])

    def LUSolve(self, B, Trans="N"):
        """Solve op(M) X = B for a vector or an N x nrhs array; returns X."""
        B = np.asarray(B)
        vec = B.ndim == 1
        X = np.array(B.reshape(self.N, -1), dtype=self.np_dtype, order="F", copy=True)
        check(lib().gbem_lu_solve(self._h, Trans.encode()[:1], X.shape[1], X.ctypes.data, self.N))
        return X[:, 0] if vec else X


class RWGGeometry:
    """Surfaces, regions and materials of a compact (non-periodic) geometry.

    surfaces: list of dicts with keys V (nv x 3), P (np x 3, 0-based), and
    material (None for PEC, a Material, or a CONST_ material name).  Region 0
    is the exterior medium (``exterior`` material, vacuum by default); each
    dielectric surface encloses its own region."""

    def __init__(self, surfaces, exterior=None, device=0):
        self.surfaces = []
        self.materials = [exterior if isinstance(exterior, Material) else (Material.parse(exterior) or Material())]
        descs = (_lib.SurfaceDesc * len(surfaces))()
        self._keep = []
        for i, s in enumerate(surfaces):
            V = np.ascontiguousarray(s["V"], dtype=np.float64)
            P = np.ascontiguousarray(s["P"], dtype=np.int32)
            mat = s.get("material")
            if isinstance(mat, str):
                mat = Material.parse(mat)
            pec = mat is None
            if not pec:
                self.materials.append(mat)
                interior = len(self.materials) - 1
            else:
                interior = -1
            self._keep += [V, P]
            descs[i] = _lib.SurfaceDesc(len(V), V.ctypes.data, len(P), P.ctypes.data, 0, interior, 1 if pec else 0)
            self.surfaces.append({"V": V, "P": P, "pec": pec, "interior": interior})
        h = ctypes.c_void_p()
        check(lib().gbem_geometry_create(len(surfaces), descs, len(self.materials), device, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_int()
        check(lib().gbem_geometry_num_bfs(h, ctypes.byref(n)))
        self.TotalBFs = n.value
        self.np_total = int(sum(len(np.asarray(d["P"])) for d in surfaces))

    @classmethod
    def from_scuffgeo(cls, path, device=0):
        """Read a .scuffgeo file with OBJECT/MESHFILE/MATERIAL/DISPLACED lines
        (RWGGeometry.cc:433-571) and CONST_ materials."""
        base = os.path.dirname(os.path.abspath(path))
        surfaces, cur = [], None
        for line in open(path):
            t = line.split("#")[0].split()
            if not t:
                continue
            kw = t[0].upper()
            if kw == "OBJECT":
                cur = {"material": None, "disp": np.zeros(3)}
            elif kw == "MESHFILE" and cur is not None:
                cur["mesh"] = os.path.join(base, t[1])
            elif kw == "MATERIAL" and cur is not None:
                cur["material"] = t[1]
            elif kw == "DISPLACED" and cur is not None:
                cur["disp"] = np.array([float(x) for x in t[1:4]])
            elif kw == "ENDOBJECT" and cur is not None:
                V, P = read_msh(cur["mesh"])
                surfaces.append({"V": V + cur["disp"], "P": P, "material": cur["material"]})
                cur = None
        return cls(surfaces, device=device)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().gbem_geometry_destroy(self._h)
            self._h = None

    def eps_mu(self, Omega):
        eps = np.array([[m.eps.real, m.eps.imag] for m in self.materials], dtype=np.float64).ravel()
        mu = np.array([[m.mu.real, m.mu.imag] for m in self.materials], dtype=np.float64).ravel()
        return eps, mu

    def edges(self, surface=0):
        n = ctypes.c_int()
        check(lib().gbem_geometry_edges(self._h, surface, ctypes.byref(n), None, None))
        E = np.zeros((n.value, 8), dtype=np.int32)
        L = np.zeros(n.value)
        check(lib().gbem_geometry_edges(self._h, surface, ctypes.byref(n), E.ctypes.data, L.ctypes.data))
        return E, L

    def cache_lookup_stats(self):
        """(hits, misses) of this geometry's near pairs in the process-wide cache."""
        h, m = ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().gbem_cache_lookup_stats(self._h, ctypes.byref(h), ctypes.byref(m)))
        return h.value, m.value

    def near_counts(self):
        c = (ctypes.c_longlong * 4)()
        check(lib().gbem_geometry_near_counts(self._h, c))
        return list(c)

    def AllocateBEMMatrix(self, dtype=C128):
        return HMatrix(self, dtype)

    def AssembleBEMMatrix(self, Omega, M=None, precision="fp64"):
        """Assemble the BEM matrix at angular frequency Omega (units of
        3e14 rad/s; lengths in microns, so the vacuum wavenumber is Omega)."""
        prec = PREC_MIXED if precision == "mixed" else PREC_FP64
        if M is None:
            M = HMatrix(self, C64 if prec == PREC_MIXED else C128)
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        check(lib().gbem_assemble(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data, prec, M._h))
        return M

    def NumBFs(self, ns):
        """Basis functions of surface ns (edges, times 2 for a dielectric)."""
        E, _ = self.edges(ns)
        return E.shape[0] * (1 if self.surfaces[ns]["pec"] else 2)

    def AssembleBEMMatrixBlock(self, nsa, nsb, Omega, M=None, RowOffset=0, ColOffset=0, real=False):
        """The (nsa, nsb) surface block (AssembleBEMMatrix.cc:349-391) written
        into the host array M (complex128, or float64 with real=True for the
        reference's real storage at imaginary frequency) at (RowOffset,
        ColOffset); allocates an NBF(nsa) x NBF(nsb) array if M is None."""
        dt = F64 if real else C128
        if M is None:
            M = np.zeros((self.NumBFs(nsa), self.NumBFs(nsb)), dtype=np.float64 if real else np.complex128, order="F")
        if not M.flags.f_contiguous:
            raise ValueError("M must be column-major (Fortran order)")
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        check(lib().gbem_assemble_block_host(self._h, nsa, nsb, Omega.real, Omega.imag, eps.ctypes.data,
                                             mu.ctypes.data, M.ctypes.data, M.shape[0], RowOffset, ColOffset, dt))
        return M

    def AssembleBEMMatrixBlockPacked(self, ns, Omega, real=False):
        """The diagonal block (ns, ns) in HMatrix's packed LHM_SYMMETRIC
        storage (upper triangle by columns, (i, j) at i + j (j+1)/2), as
        scuff-cas3D keeps its T blocks (CreateSC3Data.cc:110): a 1-D float64
        (real=True) or complex128 array of n (n + 1) / 2 entries."""
        n = self.NumBFs(ns)
        AP = np.zeros(n * (n + 1) // 2, dtype=np.float64 if real else np.complex128)
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        check(lib().gbem_assemble_block_packed_host(self._h, ns, Omega.real, Omega.imag, eps.ctypes.data,
                                                    mu.ctypes.data, AP.ctypes.data, F64 if real else C128))
        return AP

    def AssembleBEMMatrixBlockGradient(self, nsa, nsb, Omega, real=False, components=(0, 1, 2)):
        """GradM[mu] = dM_block/dx_mu for a rigid displacement of surface nsa
        (AssembleBEMMatrixBlock's GradM); returns a list of three host arrays
        (None for components not requested)."""
        dt = F64 if real else C128
        m, n = self.NumBFs(nsa), self.NumBFs(nsb)
        out = [np.zeros((m, n), dtype=np.float64 if real else np.complex128, order="F") if c in components else None
               for c in range(3)]
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        ptr = [o.ctypes.data if o is not None else None for o in out]
        check(lib().gbem_assemble_block_gradient_host(self._h, nsa, nsb, Omega.real, Omega.imag, eps.ctypes.data,
                                                      mu.ctypes.data, ptr[0], ptr[1], ptr[2], m, 0, 0, dt))
        return out

    def AssembleBEMMatrixBlockTorque(self, nsa, nsb, Omega, axes, real=False):
        """dMdT[a] = dM_block/dtheta_a for rotations of surface nsa about the
        given axes through the origin (unit vectors; AssembleBEMMatrixBlock's
        dMdT with GammaMatrix = the cross-product matrix of each axis).
        Returns a list of host arrays, one per axis."""
        axes = [np.asarray(a, dtype=np.float64) for a in axes]
        gam = np.zeros(9 * len(axes))
        for a, n in enumerate(axes):
            for nu in range(3):
                e = np.zeros(3)
                e[nu] = 1.0
                gam[9 * a + 3 * nu:9 * a + 3 * nu + 3] = np.cross(n, e)  # Gamma[mu + 3 nu] = (n x e_nu)_mu
        dt = F64 if real else C128
        m, n = self.NumBFs(nsa), self.NumBFs(nsb)
        out = [np.zeros((m, n), dtype=np.float64 if real else np.complex128, order="F") for _ in axes]
        ptrs = (ctypes.c_void_p * len(out))(*[o.ctypes.data for o in out])
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        check(lib().gbem_assemble_block_dmdt_host(self._h, nsa, nsb, Omega.real, Omega.imag, eps.ctypes.data,
                                                  mu.ctypes.data, len(axes), gam.ctypes.data, ptrs, m, 0, 0, dt))
        return out

    def GetPFT(self, Omega, KN, RHS=None, precision="fp64"):
        """Scattered and absorbed power (the reference's EMT powers, GetPFT)
        of one or more solution vectors KN (columns); RHS gives extinction.
        Returns (PAbs, PScat) arrays (PAbs is None without RHS)."""
        KN = np.asfortranarray(np.asarray(KN, dtype=np.complex128).reshape(self.TotalBFs, -1))
        nrhs = KN.shape[1]
        ps = np.zeros(nrhs)
        pe = np.zeros(nrhs)
        rp = None
        if RHS is not None:
            RHS = np.asfortranarray(np.asarray(RHS, dtype=np.complex128).reshape(self.TotalBFs, -1))
            rp = RHS.ctypes.data
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        check(lib().gbem_power_emt(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data,
                                   PREC_MIXED if precision == "mixed" else PREC_FP64, nrhs, KN.ctypes.data,
                                   self.TotalBFs, rp, self.TotalBFs, ps.ctypes.data, pe.ctypes.data))
        return (pe - ps if RHS is not None else None), ps

    def AssembleRHSVector(self, Omega, E0, nHat):
        """Plane wave E0 exp(i k nHat.x) incident from the exterior region."""
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        e0 = np.array([[complex(e).real, complex(e).imag] for e in E0], dtype=np.float64).ravel()
        nh = np.asarray(nHat, dtype=np.float64)
        out = np.zeros(self.TotalBFs, dtype=np.complex128)
        check(lib().gbem_rhs_planewave(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data,
                                       e0.ctypes.data, nh.ctypes.data, out.ctypes.data))
        return out

    @property
    def NumVertices(self):
        n = ctypes.c_int()
        check(lib().gbem_geometry_num_vertices(self._h, ctypes.byref(n)))
        return n.value

    def VertexVJPRegion(self, Omega, region, lam, x, rel_step=1e-4):
        """VertexVJP for one region's matrix alone, with exterior-region signs
        (gbem_vertex_vjp_region; region 0: the EMT power's matrix)."""
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        lam = np.asfortranarray(np.asarray(lam, dtype=np.complex128).reshape(self.TotalBFs, -1))
        x = np.asfortranarray(np.asarray(x, dtype=np.complex128).reshape(self.TotalBFs, -1))
        if lam.shape != x.shape:
            raise ValueError("lam and x need the same shape")
        g = np.zeros((self.NumVertices, 3))
        check(lib().gbem_vertex_vjp_region(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data, region,
                                           x.shape[1], lam.ctypes.data, self.TotalBFs, x.ctypes.data, self.TotalBFs,
                                           float(rel_step), g.ctypes.data))
        return g

    def ScatteredPowerGrad(self, Omega, KN):
        """dP_scat/dRe KN + i dP_scat/dIm KN per column (gbem_power_emt_grad)."""
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        KN = np.asfortranarray(np.asarray(KN, dtype=np.complex128).reshape(self.TotalBFs, -1))
        G = np.zeros_like(KN, order="F")
        check(lib().gbem_power_emt_grad(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data, KN.shape[1],
                                        KN.ctypes.data, self.TotalBFs, G.ctypes.data, self.TotalBFs))
        return G

    def VertexVJP(self, Omega, lam, x, rel_step=1e-4):
        """Re sum conj(lam) (dM/dV) x over the columns of lam and x (N x nrhs):
        the adjoint contraction with the vertex derivatives of the full BEM
        matrix, without forming them.  Returns (NumVertices, 3), surfaces'
        vertices stacked in order.  Near and common-vertex pairs take central
        differences with displacement rel_step times the pair's panel radius."""
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        lam = np.asfortranarray(np.asarray(lam, dtype=np.complex128).reshape(self.TotalBFs, -1))
        x = np.asfortranarray(np.asarray(x, dtype=np.complex128).reshape(self.TotalBFs, -1))
        if lam.shape != x.shape:
            raise ValueError("lam and x need the same shape")
        g = np.zeros((self.NumVertices, 3))
        check(lib().gbem_vertex_vjp_matrix(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data,
                                           x.shape[1], lam.ctypes.data, self.TotalBFs, x.ctypes.data, self.TotalBFs,
                                           float(rel_step), g.ctypes.data))
        return g

    def RHSVertexVJP(self, Omega, waves, gb):
        """Re sum conj(gb) (db/dV) for plane waves [(E0, nHat), ...] (the
        columns of gb, N x len(waves)).  Returns (NumVertices, 3)."""
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        gb = np.asfortranarray(np.asarray(gb, dtype=np.complex128).reshape(self.TotalBFs, -1))
        if gb.shape[1] != len(waves):
            raise ValueError("one column of gb per wave")
        e0 = np.array([[[complex(c).real, complex(c).imag] for c in E0] for E0, _ in waves], dtype=np.float64).ravel()
        nh = np.array([np.asarray(n, dtype=np.float64) for _, n in waves]).ravel()
        g = np.zeros((self.NumVertices, 3))
        check(lib().gbem_vertex_vjp_rhs_planewave(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data,
                                                  len(waves), e0.ctypes.data, nh.ctypes.data, gb.ctypes.data,
                                                  self.TotalBFs, g.ctypes.data))
        return g

    def basis_types(self):
        """Per basis function: 0 for an electric (K) current, 1 for a magnetic (N) one."""
        t = np.zeros(self.TotalBFs, dtype=np.int8)
        off = 0
        for i, s in enumerate(self.surfaces):
            ne = self.edges(i)[0].shape[0]
            if s["pec"]:
                off += ne
            else:
                t[off + 1:off + 2 * ne:2] = 1
                off += 2 * ne
        return t

    def solve_refined(self, Omega, B, tol=1e-12, max_iter=20):
        """The FP64 solve by refinement (gbem_solve_refined): FP64 matrix,
        complex64 tensor-core LU of its rounding, FP64 residuals against the
        FP64 matrix.  Returns (X, iterations, relative residual)."""
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        B = np.asfortranarray(np.asarray(B, dtype=np.complex128).reshape(self.TotalBFs, -1))
        X = np.zeros_like(B, order="F")
        it, res = ctypes.c_int(), ctypes.c_double()
        st = lib().gbem_solve_refined(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data, B.shape[1],
                                      B.ctypes.data, self.TotalBFs, X.ctypes.data, self.TotalBFs, tol, max_iter,
                                      ctypes.byref(it), ctypes.byref(res))
        if st not in (_lib.GBEM_OK, _lib.GBEM_ENOCONV):
            check(st)
        return X, it.value, res.value

    def solve_mixed(self, Omega, B, tol=1e-10, max_iter=10):
        """Mixed-precision solve (FP32 far field, complex-FP32 LU, FP64
        refinement).  Returns (X, iterations, relative residual)."""
        eps, mu = self.eps_mu(Omega)
        Omega = complex(Omega)
        B = np.asfortranarray(np.asarray(B, dtype=np.complex128).reshape(self.TotalBFs, -1))
        X = np.zeros_like(B, order="F")
        it, res = ctypes.c_int(), ctypes.c_double()
        st = lib().gbem_solve_mixed(self._h, Omega.real, Omega.imag, eps.ctypes.data, mu.ctypes.data, B.shape[1],
                                    B.ctypes.data, self.TotalBFs, X.ctypes.data, self.TotalBFs, tol, max_iter,
                                    ctypes.byref(it), ctypes.byref(res))
        if st not in (_lib.GBEM_OK, _lib.GBEM_ENOCONV):
            check(st)
        return X, it.value, res.value


def packed_dtype(AP):
    if AP.dtype == np.float64:
        return F64
    if AP.dtype == np.complex128:
        return C128
    raise ValueError("packed arrays are float64 or complex128")


def SymmetricLUFactorize(AP, N):
    """HMatrix::LUFactorize for LHM_SYMMETRIC storage (dsptrf/zsptrf 'U',
    LBWrappers.cc:159-166) on the GPU: factors the packed array AP in place
    and returns (ipiv, info) with LAPACK's pivot codes."""
    AP = np.asarray(AP)
    if not AP.flags.c_contiguous or AP.size != N * (N + 1) // 2:
        raise ValueError("AP must be a contiguous packed array of N (N + 1) / 2 entries")
    ipiv = np.zeros(N, dtype=np.int32)
    info = ctypes.c_int()
    st = lib().gbem_sp_factor_host(AP.ctypes.data, N, packed_dtype(AP), ipiv.ctypes.data, ctypes.byref(info))
    if st not in (_lib.GBEM_OK, _lib.GBEM_ESINGULAR):
        check(st)
    return ipiv, info.value


def SymmetricLUSolve(AP, N, ipiv, B):
    """HMatrix::LUSolve for LHM_SYMMETRIC storage (dsptrs/zsptrs 'U'): X with
    A X = B for the packed factor of SymmetricLUFactorize."""
    B = np.asarray(B)
    vec = B.ndim == 1
    X = np.array(B.reshape(N, -1), dtype=AP.dtype, order="F", copy=True)
    ip = np.ascontiguousarray(ipiv, dtype=np.int32)
    check(lib().gbem_sp_solve_host(AP.ctypes.data, N, packed_dtype(AP), ip.ctypes.data, X.shape[1], X.ctypes.data, N))
    return X[:, 0] if vec else X


def PreloadCache(path):
    """Load a FIPPI cache file (the reference's format, written by either
    side) into the process-wide cache (PreloadCache, libscuff.h:662)."""
    check(lib().gbem_cache_preload(os.fsencode(path)))


def StoreCache(path):
    """Write the process-wide cache -- preloaded records plus the static
    tables of every live geometry -- in the reference's format (StoreCache,
    libscuff.h:663)."""
    check(lib().gbem_cache_store(os.fsencode(path)))


def ClearCache():
    check(lib().gbem_cache_clear())


def CacheSize():
    n = ctypes.c_longlong()
    check(lib().gbem_cache_size(ctypes.byref(n)))
    return n.value


def LUTuning(device=0):
    """The LU tuning choices made so far on a device (gbem_lu_tuning): the
    register leaf's threads per rows-per-CTA bucket and the complex-FP32 panel
    width per N bucket, as a dict."""
    import json
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib().gbem_lu_tuning(int(device), buf, len(buf)))
    return json.loads(buf.value.decode())


def solve_mixed_batch(jobs, max_concurrent=4, tol=1e-10, max_iter=10):
    """Independent mixed-precision solves run as one batch
    (gbem_solve_mixed_batch): jobs is a list of (RWGGeometry, Omega, B);
    up to max_concurrent at once, each on its geometry's stream from its own
    host thread, jobs on one geometry in turn, largest N first.  Returns
    [(X, iterations, relative residual)] in job order."""
    arr = (_lib.BatchJob * len(jobs))()
    keep = []
    for j, (G, Omega, B) in enumerate(jobs):
        eps, mu = G.eps_mu(Omega)
        Omega = complex(Omega)
        B = np.asfortranarray(np.asarray(B, dtype=np.complex128).reshape(G.TotalBFs, -1))
        X = np.zeros_like(B, order="F")
        keep.append((eps, mu, B, X))
        arr[j].g = G._h
        arr[j].omega_re, arr[j].omega_im = Omega.real, Omega.imag
        arr[j].eps, arr[j].mu = eps.ctypes.data, mu.ctypes.data
        arr[j].nrhs = B.shape[1]
        arr[j].B, arr[j].ldb = B.ctypes.data, G.TotalBFs
        arr[j].X, arr[j].ldx = X.ctypes.data, G.TotalBFs
        arr[j].tol, arr[j].max_iter = tol, max_iter
    st = lib().gbem_solve_mixed_batch(len(jobs), arr, max_concurrent)
    if st not in (_lib.GBEM_OK, _lib.GBEM_ENOCONV):
        check(st)
    return [(keep[j][3], arr[j].iters, arr[j].resid) for j in range(len(jobs))]

