"""The scuff-cas3D per-frequency Casimir integrand on the GPU.

For compact geometries at imaginary frequency Omega = i xi the BEM matrix is
real; the reference forms (applications/scuff-cas3D/CasimirIntegrand.cc):

* energy integrand  -1/(2 pi) log |det M_inf / det M|, with det M_inf the
  product of the diagonal blocks' determinants (the T blocks, factored on
  their own; CasimirIntegrand.cc:50-63, 296-358),
* z-force integrand  -1/(2 pi) * 2 * Tr[M^-1 dM], where dM (N x N1) holds the
  transposes of dU/dz, the derivatives of the U(0, s) blocks under a rigid
  displacement of surface 0, at rows of surface s (CasimirIntegrand.cc:100-146,
  441-452).

Here M, the T blocks and dU/dz are assembled on the GPU (gbem_assemble and
gbem_assemble_block_gradient in real storage), factored there
(gbem_lu_factor), and log|det| and the trace are reduced there
(gbem_lu_log_abs_det, gbem_lu_trace_host).
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import F64
from .api import HMatrix, RWGGeometry


def laguerre_xi(n=20, gap=1.0):
    """Nodes and weights of the n-point Gauss-Laguerre rule for
    int_0^inf f(xi) dxi with xi = x / gap: xi_j = x_j / gap and weights
    w_j e^{x_j} / gap, so that sum_j W_j f(xi_j) approximates the integral."""
    x, w = np.polynomial.laguerre.laggauss(n)
    return x / gap, w * np.exp(x) / gap


class CasimirIntegrand:
    """Energy and z-force integrands of the bodies of ``surfaces`` (a list of
    gbem surface dicts; PEC when ``material`` is None) at imaginary
    frequencies.  Bodies whose meshes are translates of an earlier body's
    share its T-block factor, as the reference's mates do (Mate[],
    CasimirIntegrand.cc:290-296)."""

    def __init__(self, surfaces, device=0):
        self.surfaces = surfaces
        self.G = RWGGeometry(surfaces, device=device)
        self.N = self.G.TotalBFs
        self.nbf = [self.G.NumBFs(s) for s in range(len(surfaces))]
        self.offset = np.concatenate([[0], np.cumsum(self.nbf)]).astype(int)
        # one single-body geometry per distinct body (translates share)
        self._mate, self._single = [], {}
        for s, d in enumerate(surfaces):
            m = self._find_mate(s)
            self._mate.append(m)
            if m == s:
                self._single[s] = RWGGeometry([d], device=device)

    def _find_mate(self, s):
        d = self.surfaces[s]
        V, P = np.asarray(d["V"]), np.asarray(d["P"])
        for t in range(s):
            e = self.surfaces[t]
            Vt, Pt = np.asarray(e["V"]), np.asarray(e["P"])
            if Pt.shape == P.shape and np.array_equal(Pt, P) and d.get("material") == e.get("material"):
                shift = V[0] - Vt[0]
                if np.array_equal(Vt + shift, V):
                    return self._mate[t]
        return s

    def log_abs_det_blocks(self, xi):
        """sum over bodies of log|det T_s| at Omega = i xi."""
        tot, memo = 0.0, {}
        for s in range(len(self.surfaces)):
            m = self._mate[s]
            if m not in memo:
                Gs = self._single[m]
                T = Gs.AssembleBEMMatrix(1j * xi, HMatrix(Gs, F64))
                T.LUFactorize()
                memo[m] = T.LogAbsDet()
            tot += memo[m]
        return tot

    def __call__(self, xi, energy=True, zforce=True):
        """(energy integrand, z-force integrand) at Omega = i xi; None for a
        quantity not requested."""
        M = self.G.AssembleBEMMatrix(1j * xi, HMatrix(self.G, F64))
        M.LUFactorize()
        E = F = None
        if energy:
            ld = self.log_abs_det_blocks(xi) - M.LogAbsDet()
            E = -ld / (2.0 * math.pi) if math.isfinite(ld) else 0.0
        if zforce:
            N1 = self.nbf[0]
            dM = np.zeros((self.N, N1), dtype=np.float64, order="F")
            for s in range(1, len(self.surfaces)):
                g = self.G.AssembleBEMMatrixBlockGradient(0, s, 1j * xi, real=True, components=(2,))[2]
                o = self.offset[s]
                dM[o:o + self.nbf[s], :] = g.T
            tr = 2.0 * M.TraceMInvdM(dM, N1).real
            F = -tr / (2.0 * math.pi) if math.isfinite(tr) else 0.0
        return E, F
