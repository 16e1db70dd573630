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
