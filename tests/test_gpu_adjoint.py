"""Shape derivatives through the adjoint (gbem.adjoint): the autograd
gradient of the extinction power with respect to the vertex positions
against central finite differences of the GPU forward solve, its translation
invariance, and the mixed-precision form against the FP64 one.  The
reference has no shape derivative (only rigid-motion GradM/dMdT), so the
forward model itself is the oracle here."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WAVES = [((1, 0, 0), (0, 0, 1)), ((0, 1, 0), (-0.6, 0, 0.8))]


def _case(kind, subdiv=1):
    from gbem import mesh
    from gbem.adjoint import MeshTopology
    from gbem.api import Material
    V, P = mesh.icosphere(subdiv)
    if kind == "pec":
        surfs, w = [{"V": V, "P": P, "material": None}], 1.0
    elif kind == "diel":
        surfs, w = [{"V": V, "P": P, "material": Material(2.25 + 0.01j)}], 2.0
    else:  # a PEC and a lossy dielectric sphere 0.6 apart: the inter-surface blocks
        surfs = [{"V": V, "P": P, "material": None},
                 {"V": 0.8 * V + np.array([0.3, 0.0, 2.4]), "P": P, "material": Material(4.0 + 0.2j)}]
        w = 1.5
    return MeshTopology.from_surfaces(surfs) + (w,)


def _power(topo, V, w, precision="fp64", grad=True):
    import torch
    from gbem.adjoint import extinction_power, scatter
    Vt = torch.tensor(V, dtype=torch.float64, requires_grad=grad)
    x, b = scatter(Vt, topo, w, WAVES, precision=precision)
    types = topo.geometry(V).basis_types()
    p = extinction_power(x, b, types).sum()
    if not grad:
        return float(p)
    p.backward()
    return float(p), Vt.grad.numpy().copy()


@pytest.mark.parametrize("kind", ["pec", "diel", "two"])
def test_extinction_gradient_matches_central_differences(kind):
    topo, V0, w = _case(kind)
    p0, g = _power(topo, V0, w)
    assert p0 > 0
    rng = np.random.default_rng(0)
    picks = rng.choice(V0.size, size=10, replace=False)
    h = 1e-5
    err = 0.0
    for q in picks:
        Vp, Vm = V0.copy(), V0.copy()
        Vp.flat[q] += h
        Vm.flat[q] -= h
        fd = (_power(topo, Vp, w, grad=False) - _power(topo, Vm, w, grad=False)) / (2 * h)
        err = max(err, abs(fd - g.flat[q]))
    rel = err / np.abs(g).max()
    print("%s: P_ext %.6e, |g|max %.3e, max |fd - adjoint| / |g|max = %.2e" % (kind, p0, np.abs(g).max(), rel))
    assert rel < 1e-5


def test_gradient_is_translation_invariant():
    """The power does not change when the whole scatterer moves, so the
    vertex gradients sum to zero, on a larger mesh (icosphere s=3, N = 3840):
    a check of the far pairs' reverse-mode derivative against the right-hand
    side's (the near pairs use the same invariance to skip one vertex each)."""
    topo, V0, w = _case("diel", subdiv=3)
    t0 = time.perf_counter()
    p0, g = _power(topo, V0, w)
    dt = time.perf_counter() - t0
    s = np.abs(g.sum(axis=0)).max() / np.abs(g).sum(axis=0).max()
    print("s=3: P_ext %.6e, forward+backward %.2f s, |sum g| / sum |g| = %.2e" % (p0, dt, s))
    assert s < 1e-8


def test_mixed_gradient_matches_fp64():
    topo, V0, w = _case("diel", subdiv=2)
    p64, g64 = _power(topo, V0, w, precision="fp64")
    p32, g32 = _power(topo, V0, w, precision="mixed")
    assert abs(p32 - p64) / abs(p64) < 1e-6
    rel = np.abs(g32 - g64).max() / np.abs(g64).max()
    print("mixed vs fp64 gradient: %.2e" % rel)
    assert rel < 1e-5


def test_vertex_gradient_sums_to_the_rigid_displacement_gradient():
    """Summed over one body's vertices, the vertex contraction is the
    derivative under a rigid displacement of that body -- the reference's own
    dM/dx_mu force path (AssembleBEMMatrixBlock's GradM, pinned against the
    reference in test_gpu_gradient.py).  Bodies 2.2 apart: every inter-body
    pair is a far pair, where both use the 6x6 rule, so they agree to rounding."""
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(1)
    G = RWGGeometry([{"V": V, "P": P, "material": None},
                     {"V": 0.8 * V + np.array([0.3, 0.0, 4.0]), "P": P, "material": Material(4.0 + 0.2j)}])
    w = 1.5
    N, n0 = G.TotalBFs, G.NumBFs(0)
    rng = np.random.default_rng(3)
    # lam only on body 1's rows and x only on body 0's: the self blocks drop out
    # (their translation-invariant terms would cancel only to the near pairs'
    # difference accuracy, ~1e-7 of this weak inter-body term)
    lam = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    x = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    lam[:n0] = 0.0
    x[n0:] = 0.0
    g = G.VertexVJP(w, lam, x)
    rigid = g[len(V):].sum(axis=0)
    D = G.AssembleBEMMatrixBlockGradient(1, 0, w)  # block (1, 0), surface 1 displaced
    ref = np.array([np.real(np.sum(np.conj(lam[n0:]) * (D[m] @ x[:n0]))) for m in range(3)])
    rel = np.abs(rigid - ref).max() / np.abs(ref).max()
    print("sum of vertex gradients vs GradM contraction: %.2e" % rel)
    assert rel < 1e-9


def _absorbed(topo, V, w, waves, precision="fp64", grad=True):
    import torch
    from gbem.adjoint import absorbed_power, scatter
    Vt = torch.tensor(V, dtype=torch.float64, requires_grad=grad)
    x, b = scatter(Vt, topo, w, waves, precision=precision)
    p = absorbed_power(x, b, Vt, topo, w).sum()
    if not grad:
        return float(p)
    p.backward()
    return float(p), Vt.grad.numpy().copy()


@pytest.mark.parametrize("kind", ["diel", "two"])
def test_absorbed_power_gradient_matches_central_differences(kind):
    """Absorbed power = extinction - EMT scattered power, whose scattered
    part depends on the vertices through the exterior region's matrix too
    (gbem_vertex_vjp_region, gbem_power_emt_grad)."""
    topo, V0, w = _case(kind)
    p0, g = _absorbed(topo, V0, w, WAVES)
    assert p0 > 0
    rng = np.random.default_rng(1)
    picks = rng.choice(V0.size, size=10, replace=False)
    h = 1e-5
    err = 0.0
    for q in picks:
        Vp, Vm = V0.copy(), V0.copy()
        Vp.flat[q] += h
        Vm.flat[q] -= h
        fd = (_absorbed(topo, Vp, w, WAVES, grad=False) - _absorbed(topo, Vm, w, WAVES, grad=False)) / (2 * h)
        err = max(err, abs(fd - g.flat[q]))
    rel = err / np.abs(g).max()
    print("%s: P_abs %.6e, |g|max %.3e, max |fd - adjoint| / |g|max = %.2e" % (kind, p0, np.abs(g).max(), rel))
    assert rel < 1e-5


def _far_flags(V, P, panels):
    """rRel > 4 (the far-pair test of AssessPanelPair.cc:52-103: centroid
    distance over the larger panel radius) of the given panels against every
    panel."""
    c = V[P].mean(axis=1)
    r = np.max(np.linalg.norm(V[P] - c[:, None, :], axis=2), axis=1)
    d = np.linalg.norm(c[panels][:, None, :] - c[None, :, :], axis=2)
    return d / np.maximum(r[panels][:, None], r[None, :]) > 4.0


def test_absorbed_power_gradient_2562_vertices():
    """The shape gradient at the benchmark's size: the dielectric sphere
    (eps = 2.25+0.01i, icosphere s=4: 2562 vertices, N = 15360) at kR = 2,
    absorbed power of one plane wave, against central differences with step
    1e-4 along one seeded random direction at each of 32 seeded vertices.
    Forward solves by FP64 refinement (gbem_solve_refined) so the differences
    see the FP64 model; gate 1e-5 of the gradient's largest component.

    The discretised model is smooth in the vertices only piecewise: a panel
    pair is integrated by the 6x6 rule when rRel > 4 and by the near-pair
    scheme otherwise (the reference's own switch, PanelPanelInteractions.cc:
    357-561), and a step that carries a pair across rRel = 4 differences two
    branches.  Vertices whose +-h step moves any of their panels' pairs across
    the switch are passed over (the next seeded vertex is taken)."""
    from gbem import mesh
    from gbem.adjoint import MeshTopology
    from gbem.api import Material
    V, P = mesh.icosphere(4)
    topo, V0 = MeshTopology.from_surfaces([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}])
    w = 2.0
    waves = WAVES[:1]
    t0 = time.perf_counter()
    p0, g = _absorbed(topo, V0, w, waves, precision="refined")
    t_grad = time.perf_counter() - t0
    rng = np.random.default_rng(0)
    order = rng.permutation(len(V0))
    h = 1e-4
    worst, used, skipped = 0.0, 0, 0
    t0 = time.perf_counter()
    for v in order:
        if used == 32:
            break
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        Vp, Vm = V0.copy(), V0.copy()
        Vp[v] += h * d
        Vm[v] -= h * d
        panels = np.nonzero((P == v).any(axis=1))[0]
        if not np.array_equal(_far_flags(Vp, P, panels), _far_flags(Vm, P, panels)):
            skipped += 1
            continue
        fd = (_absorbed(topo, Vp, w, waves, "refined", grad=False) -
              _absorbed(topo, Vm, w, waves, "refined", grad=False)) / (2 * h)
        worst = max(worst, abs(fd - g[v] @ d))
        used += 1
    rel = worst / np.abs(g).max()
    print("s=4: P_abs %.6e, |g|max %.3e, gradient %.1f s, %d vertices (%d passed over at the rRel = 4 switch), "
          "FD solves %.1f s, max |fd - adjoint| / |g|max = %.2e"
          % (p0, np.abs(g).max(), t_grad, used, skipped, time.perf_counter() - t0, rel))
    assert used == 32
    assert rel < 1e-5
