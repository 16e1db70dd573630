"""GPU assembly (through the C ABI) against the oracle and the reference."""
import numpy as np
import pytest

from helpers import fixture_surfaces, omega_of, relerr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ora():
    from oracle import oracle
    return oracle


@pytest.mark.parametrize("case", ["diel_s1_w2", "pec2_s1_xi", "pec_s2_w1"])
def test_fp64_matches_reference_and_oracle(golden, ora, case):
    from gbem import RWGGeometry
    d = golden("ref_%s.npz" % case)
    gs, (regs, pec, eps, mu) = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    M = G.AssembleBEMMatrix(w).numpy()
    osurf = [ora.Surface(s["V"], s["P"]) for s in gs]
    Mo = ora.assemble(osurf, regs, pec, w, eps, mu)
    # GPU vs oracle: both integrate near pairs far below the reference's tolerance
    assert relerr(M, Mo) < 1e-11, relerr(M, Mo)
    assert np.array_equal(M, M.T)
    if "M" in d.files:
        assert relerr(M, d["M"]) < 2e-7
    else:
        assert relerr(M[:, d["cols"]], d["Mcols"]) < 2e-7


def test_far_entries_bitwise_formula(golden, ora):
    """Entries whose panel pairs are all far (6x6 rule) agree with the
    reference to rounding: the same 13-digit rule, the same kernel."""
    from gbem import RWGGeometry
    d = golden("ref_pec_s2_w1.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    M = G.AssembleBEMMatrix(omega_of(d)).numpy()
    cols = d["cols"]
    Mr = d["Mcols"]
    E, _ = G.edges(0)
    V, P = gs[0]["V"], gs[0]["P"]
    c = V[P].mean(axis=1)
    r = np.max(np.linalg.norm(V[P] - c[:, None, :], axis=2), axis=1)
    worst = 0.0
    scale = np.abs(Mr).max()
    for j, col in enumerate(cols):
        pj = [E[col, 4], E[col, 5]]
        for i in range(480):
            pi = [E[i, 4], E[i, 5]]
            if all(np.linalg.norm(c[a] - c[b]) / max(r[a], r[b]) > 4.0 for a in pi for b in pj):
                # a few entries vanish by the mesh's symmetry: floor the scale
                worst = max(worst, abs(M[i, col] - Mr[i, j]) / max(abs(Mr[i, j]), 1e-6 * scale))
    assert worst < 1e-10, worst


def test_mixed_precision_far_field(golden):
    from gbem import RWGGeometry
    d = golden("ref_diel_s1_w2.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    M64 = G.AssembleBEMMatrix(w).numpy()
    M32 = G.AssembleBEMMatrix(w, precision="mixed").numpy()
    assert M32.dtype == np.complex64
    err = np.abs(M32.astype(np.complex128) - M64)
    assert err.max() / np.abs(M64).max() < 2e-6
    assert np.linalg.norm(err) / np.linalg.norm(M64) < 1e-6


def test_larger_dielectric_against_oracle(ora):
    """Subdivision-2 dielectric sphere (N = 960), eps = 2.25+0.01i, kR = 2."""
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(2)
    m = Material(2.25 + 0.01j)
    G = RWGGeometry([{"V": V, "P": P, "material": m}])
    M = G.AssembleBEMMatrix(2.0).numpy()
    Mo = ora.assemble([ora.Surface(V, P)], [(0, 1)], [False], 2.0, [1.0, m.eps], [1.0, 1.0])
    assert relerr(M, Mo) < 1e-11


def test_short_wavelength_touching_pairs_report_enotsup(golden):
    from gbem import GbemError, RWGGeometry
    d = golden("ref_diel_s1_w12.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    with pytest.raises(GbemError) as e:
        G.AssembleBEMMatrix(omega_of(d))
    assert "ENOTSUP" in str(e.value)
