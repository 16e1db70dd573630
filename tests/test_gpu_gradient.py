"""Gradient blocks dM/dx_mu (AssembleBEMMatrixBlock's GradM, the cas3D force
path) against the reference and against finite differences."""
import numpy as np
import pytest

from helpers import fixture_surfaces, omega_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,blocks", [("pec2_s1_grad", [(0, 1), (1, 0)]), ("diel2_s1_grad", [(0, 1)])])
def test_far_block_gradients_match_reference(golden, case, blocks):
    """Inter-sphere blocks (centre gap 3: far pairs on the 6x6 rule, the
    nearest pairs on the high-order rule with smooth integrands): the
    gradients agree with the reference to ~1e-11; the block itself carries the
    usual desingularised near-pair difference (~1e-9)."""
    from gbem import RWGGeometry
    d = golden("ref_%s.npz" % case)
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    for (a, b) in blocks:
        M = G.AssembleBEMMatrixBlock(a, b, w)
        assert np.abs(M - d["M%d%d" % (a, b)]).max() <= 2e-7 * np.abs(d["M%d%d" % (a, b)]).max()
        grads = G.AssembleBEMMatrixBlockGradient(a, b, w)
        ref = d["G%d%d" % (a, b)]
        for mu in range(3):
            err = np.abs(grads[mu] - ref[mu]).max() / np.abs(ref[mu]).max()
            assert err < 1e-10, (a, b, mu, err)


def test_gradient_matches_finite_differences(golden):
    """dU/dz of the inter-sphere block against central differences of the
    assembled block under a displacement of sphere 0 (step 1e-4).  The block
    desingularises its near pairs while the gradient integrates them directly
    (as the reference does), so they agree to ~3e-6, as the reference's own
    gradient does."""
    from gbem import RWGGeometry
    d = golden("ref_diel2_s1_grad.npz")
    gs, _ = fixture_surfaces(d)
    w = omega_of(d)
    h = 1e-4
    Ms = []
    for sgn in (+1, -1):
        g2 = [dict(s) for s in gs]
        g2[0]["V"] = gs[0]["V"] + np.array([0.0, 0.0, sgn * h])
        Ms.append(RWGGeometry(g2).AssembleBEMMatrixBlock(0, 1, w))
    fd = (Ms[0] - Ms[1]) / (2 * h)
    gz = RWGGeometry(gs).AssembleBEMMatrixBlockGradient(0, 1, w, components=(2,))[2]
    assert np.abs(gz - fd).max() / np.abs(gz).max() < 1e-5


def test_real_storage_and_skipped_components(golden):
    """F64 gradients at imaginary frequency are the real parts; components not
    asked for are not computed."""
    from gbem import RWGGeometry
    d = golden("ref_pec2_s1_grad.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    full = G.AssembleBEMMatrixBlockGradient(0, 1, w)
    real = G.AssembleBEMMatrixBlockGradient(0, 1, w, real=True, components=(2,))
    assert real[0] is None and real[1] is None
    assert np.array_equal(real[2], full[2].real)
    assert np.abs(full[2].imag).max() <= 1e-14 * np.abs(full[2]).max()


@pytest.mark.parametrize("real", [False, True])
def test_casimir_trace_matches_reference_and_log_det(golden, real):
    """Tr[M^-1 dM/dz] (GetTraceMInvdM, CasimirIntegrand.cc:100-146) on the GPU:
    the block column [0; dU01^T] of a displacement of sphere 0, traced over
    sphere 0's basis functions.  It matches the same trace formed from the
    reference's own matrix and gradient, and twice it is d(log det M)/dz by
    central differences (step 1e-4), since dM/dz = [[0, dU], [dU^T, 0]] for a
    rigid displacement and M is symmetric."""
    from gbem import C128, F64, RWGGeometry
    from gbem.api import HMatrix
    d = golden("ref_pec2_s1_grad.npz")
    dx = golden("ref_pec2_s1_xi.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    N0 = G.NumBFs(0)
    Mc = G.AssembleBEMMatrix(w).numpy()
    N = Mc.shape[0]
    dU = G.AssembleBEMMatrixBlockGradient(0, 1, w, real=real, components=(2,))[2]
    B = np.zeros((N, N0), dtype=np.float64 if real else np.complex128)
    B[N0:, :] = dU.T
    M = HMatrix(G, F64 if real else C128)
    M.set(Mc.real if real else Mc)
    assert M.LUFactorize() == 0
    tr = M.TraceMInvdM(B)
    # the same trace from the reference's matrix and gradient
    Br = np.zeros((N, N0), dtype=np.complex128)
    Br[N0:, :] = d["G01"][2].T
    Xr = np.linalg.solve(dx["M"], Br)
    tr_ref = np.trace(Xr[:N0, :N0])
    assert abs(tr - tr_ref) < 1e-8 * abs(tr_ref), (tr, tr_ref)
    # and the derivative of log det M
    h = 1e-4
    ld = []
    for sgn in (+1, -1):
        g2 = [dict(s) for s in gs]
        g2[0]["V"] = gs[0]["V"] + np.array([0.0, 0.0, sgn * h])
        ld.append(np.linalg.slogdet(RWGGeometry(g2).AssembleBEMMatrix(w).numpy())[1])
    fd = (ld[0] - ld[1]) / (2 * h)
    assert abs(2 * tr.real - fd) < 1e-5 * abs(fd), (2 * tr.real, fd)


@pytest.mark.parametrize("case,blocks", [("pec2_s1_torque", [(0, 1), (1, 0)]), ("diel2_s1_torque", [(0, 1)])])
def test_torque_blocks_match_reference(golden, case, blocks):
    """dM/dtheta for rotations of the row surface about the x, y, z axes
    through the origin (AssembleBEMMatrixBlock's dMdT with GammaMatrix, the
    scuff-cas3D torque path) against the reference."""
    from gbem import RWGGeometry
    d = golden("ref_%s.npz" % case)
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    for (a, b) in blocks:
        T = G.AssembleBEMMatrixBlockTorque(a, b, w, np.eye(3))
        ref = d["T%d%d" % (a, b)]
        for ax in range(3):
            err = np.abs(T[ax] - ref[ax]).max() / np.abs(ref).max()
            assert err < 1e-10, (a, b, ax, err)
    if d["omega"][0] == 0.0:  # imaginary frequency: real storage gives the real parts
        Tr = G.AssembleBEMMatrixBlockTorque(0, 1, w, [(0.0, 0.0, 1.0)], real=True)[0]
        assert np.abs(Tr - d["T01"][2].real).max() < 1e-10 * np.abs(d["T01"][2]).max()


def test_torque_matches_finite_differences(golden):
    """dU/dtheta_z of the inter-sphere block against central differences under
    a rotation of sphere 0 about the z axis (step 1e-4 rad)."""
    from gbem import RWGGeometry
    d = golden("ref_diel2_s1_torque.npz")
    gs, _ = fixture_surfaces(d)
    w = omega_of(d)
    h = 1e-4
    Ms = []
    for sgn in (+1, -1):
        c, s = np.cos(sgn * h), np.sin(sgn * h)
        Rz = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
        g2 = [dict(x) for x in gs]
        g2[0]["V"] = gs[0]["V"] @ Rz.T
        Ms.append(RWGGeometry(g2).AssembleBEMMatrixBlock(0, 1, w))
    fd = (Ms[0] - Ms[1]) / (2 * h)
    tz = RWGGeometry(gs).AssembleBEMMatrixBlockTorque(0, 1, w, [(0.0, 0.0, 1.0)])[0]
    assert np.abs(tz - fd).max() / np.abs(tz).max() < 1e-5
