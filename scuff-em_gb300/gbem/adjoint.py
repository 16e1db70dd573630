"""Shape derivatives through PyTorch autograd.

``scatter(V, topology, Omega, waves)`` solves the plane-wave scattering
problem M(V) x = b(V) for the vertex positions V (a float64 tensor, all
surfaces' vertices stacked) and returns the surface currents x and the
right-hand sides b (N x nwaves, complex128) as differentiable functions of V.
Any real loss built from x and b (``extinction_power`` below, for one)
back-propagates to V through one adjoint solve,

    lam = M^-H dL/dx,    dL/dV = -Re lam^H (dM/dV) x + Re (lam + dL/db)^H (db/dV),

whose two contractions run on the GPU (``RWGGeometry.VertexVJP`` and
``RWGGeometry.RHSVertexVJP``) without forming dM/dV.  The matrix is complex
symmetric (M^T = M, AssembleBEMMatrix.cc:753-758), so M^-H g = conj(M^-1
conj(g)) reuses the forward factorisation.

The reference has no shape derivative: its GradM/dMdT blocks differentiate
rigid motions of whole surfaces (libscuff.h:500-505).
"""
from __future__ import annotations

import numpy as np
import torch

from .api import ZVAC, RWGGeometry


class MeshTopology:
    """The fixed part of a geometry: per surface its panels (np x 3, 0-based
    vertex indices) and material (None = PEC); vertex positions come later."""

    def __init__(self, surfaces, exterior=None, device=0):
        self.surfaces = [{"P": np.asarray(s["P"], dtype=np.int32), "material": s.get("material"),
                          "nv": int(s["nv"])} for s in surfaces]
        self.exterior = exterior
        self.device = device

    @classmethod
    def from_surfaces(cls, surfaces, exterior=None, device=0):
        """From RWGGeometry-style dicts (V, P, material); returns (topology, V0)."""
        topo = cls([{"P": s["P"], "material": s.get("material"), "nv": len(s["V"])} for s in surfaces],
                   exterior, device)
        return topo, np.concatenate([np.asarray(s["V"], dtype=np.float64) for s in surfaces])

    @property
    def num_vertices(self):
        return sum(s["nv"] for s in self.surfaces)

    def geometry(self, V):
        V = np.asarray(V, dtype=np.float64).reshape(-1, 3)
        if V.shape[0] != self.num_vertices:
            raise ValueError("V has %d vertices, the topology %d" % (V.shape[0], self.num_vertices))
        out, off = [], 0
        for s in self.surfaces:
            out.append({"V": V[off:off + s["nv"]], "P": s["P"], "material": s["material"]})
            off += s["nv"]
        return RWGGeometry(out, exterior=self.exterior, device=self.device)


class _Scatter(torch.autograd.Function):
    @staticmethod
    def forward(ctx, V, topology, Omega, waves, precision, rel_step):
        geo = topology.geometry(V.detach().cpu().numpy())
        b = np.stack([geo.AssembleRHSVector(Omega, E0, nh) for E0, nh in waves], axis=1)
        if precision == "fp64":
            M = geo.AssembleBEMMatrix(Omega)
            if M.LUFactorize() != 0:
                raise RuntimeError("singular BEM matrix")
            x = M.LUSolve(b)
            solve = M.LUSolve
        elif precision == "mixed":
            x = geo.solve_mixed(Omega, b)[0]
            solve = lambda B: geo.solve_mixed(Omega, B)[0]  # noqa: E731
        elif precision == "refined":
            # the FP64 solution by mixed-precision refinement against the FP64 matrix
            x = geo.solve_refined(Omega, b)[0]
            solve = lambda B: geo.solve_refined(Omega, B)[0]  # noqa: E731
        else:
            raise ValueError("precision must be 'fp64', 'mixed' or 'refined'")
        ctx.geo, ctx.solve, ctx.Omega, ctx.waves, ctx.rel_step = geo, solve, Omega, waves, rel_step
        ctx.x = x
        ctx.vdevice, ctx.vdtype = V.device, V.dtype
        return torch.from_numpy(np.ascontiguousarray(x)), torch.from_numpy(np.ascontiguousarray(b))

    @staticmethod
    def backward(ctx, gx, gb):
        x = ctx.x
        gx = np.zeros_like(x) if gx is None else gx.detach().resolve_conj().cpu().numpy().astype(np.complex128)
        gb = np.zeros_like(x) if gb is None else gb.detach().resolve_conj().cpu().numpy().astype(np.complex128)
        # lam = M^-H gx = conj(M^-1 conj(gx))  (M complex symmetric)
        lam = np.conj(ctx.solve(np.conj(gx)))
        g = -ctx.geo.VertexVJP(ctx.Omega, lam, x, rel_step=ctx.rel_step)
        g += ctx.geo.RHSVertexVJP(ctx.Omega, ctx.waves, lam + gb)
        return torch.from_numpy(g).to(device=ctx.vdevice, dtype=ctx.vdtype), None, None, None, None, None


def scatter(V, topology, Omega, waves, precision="fp64", rel_step=1e-4):
    """(x, b) for plane waves [(E0, nHat), ...] incident from the exterior
    region, differentiable with respect to the vertex tensor V (nv x 3)."""
    return _Scatter.apply(V, topology, complex(Omega), [(tuple(E0), tuple(nh)) for E0, nh in waves], precision,
                          rel_step)


class _ScatteredPower(torch.autograd.Function):
    """EMT scattered power of the solutions x (one value per column) as a
    function of x and of the vertices V (the exterior region's matrix in its
    quadratic form depends on V)."""

    @staticmethod
    def forward(ctx, x, V, topology, Omega, rel_step):
        geo = topology.geometry(V.detach().cpu().numpy())
        xn = x.detach().resolve_conj().cpu().numpy().astype(np.complex128)
        _, ps = geo.GetPFT(Omega, xn)
        ctx.geo, ctx.Omega, ctx.rel_step, ctx.x = geo, Omega, rel_step, xn
        ctx.vdevice, ctx.vdtype = V.device, V.dtype
        return torch.from_numpy(np.asarray(ps, dtype=np.float64)).to(x.device)

    @staticmethod
    def backward(ctx, gp):
        geo, x = ctx.geo, ctx.x
        w = gp.detach().cpu().numpy().astype(np.float64)
        gx = geo.ScatteredPowerGrad(ctx.Omega, x) * w[None, :]
        # explicit part: P = 1/2 sum Re(w_ij M0_ij) with M0 the exterior
        # region's matrix; w = conj(l1) x1^T + conj(l2) x2^T with c = D x
        # (D = 1 on K rows, -ZVAC on N rows):
        #   l1 = p c, x1 = q c, l2 = p' conj(c), x2 = q' conj(c),
        #   p = (1, 1/ZVAC), q = (-ZVAC/2, 1/2), p' = (1, -1/ZVAC), q' = (-ZVAC/2, -1/2) on (K, N) rows
        nrow = np.asarray(geo.basis_types()) == 1
        d = np.where(nrow, -ZVAC, 1.0)[:, None]
        c = d * x
        p = np.where(nrow, 1.0 / ZVAC, 1.0)[:, None]
        q = np.where(nrow, 0.5, -0.5 * ZVAC)[:, None]
        pp = np.where(nrow, -1.0 / ZVAC, 1.0)[:, None]
        qq = np.where(nrow, -0.5, -0.5 * ZVAC)[:, None]
        lam = np.concatenate([p * c * w[None, :], pp * np.conj(c) * w[None, :]], axis=1)
        xx = np.concatenate([q * c, qq * np.conj(c)], axis=1)
        gV = 0.5 * geo.VertexVJPRegion(ctx.Omega, 0, lam, xx, rel_step=ctx.rel_step)
        return (torch.from_numpy(gx), torch.from_numpy(gV).to(device=ctx.vdevice, dtype=ctx.vdtype), None, None,
                None)


def scattered_power(x, V, topology, Omega, rel_step=1e-4):
    """EMT scattered power per column of x (the reference's default power
    method, GetPFT with EMT, EMTPFT.cc:642-700), differentiable with respect
    to x and to the vertex tensor V."""
    return _ScatteredPower.apply(x, V, topology, complex(Omega), rel_step)


def absorbed_power(x, b, V, topology, Omega, rel_step=1e-4):
    """Absorbed power per column: extinction minus scattered power (the
    reference's EMT split, EMTPFT.cc:305-392), differentiable with respect to
    the solutions, the right-hand sides and the vertices."""
    types = topology.geometry(V.detach().cpu().numpy()).basis_types()
    return extinction_power(x, b, types) - scattered_power(x, V, topology, Omega, rel_step)


def extinction_power(x, b, types):
    """Extinction power per wave, -1/2 ZVAC sum_i s_i Re(conj(x_i) b_i) with
    s_i = -1 on magnetic (N) rows (the reference's EMT extinction,
    EMTPFT.cc:305-392); ``types`` from ``RWGGeometry.basis_types()``."""
    s = torch.from_numpy(np.where(np.asarray(types) == 1, -1.0, 1.0)).to(x.device)
    return -0.5 * ZVAC * (s[:, None] * (torch.conj(x) * b).real).sum(dim=0)
