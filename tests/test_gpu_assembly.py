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


def test_short_wavelength_touching_pairs(golden, ora):
    """eps = 4+0.1i at kR = 12: |k r| > pi on the touching pairs, which take the
    full-kernel Taylor-Duffy branch (PanelPanelInteractions.cc:449-491)."""
    from gbem import RWGGeometry
    d = golden("ref_diel_s1_w12.npz")
    gs, (regs, pec, eps, mu) = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    M = G.AssembleBEMMatrix(w).numpy()
    Mo = ora.assemble([ora.Surface(s["V"], s["P"]) for s in gs], regs, pec, w, eps, mu)
    assert np.array_equal(M, M.T)
    assert relerr(M, Mo) < 1e-9, relerr(M, Mo)
    # the reference caps its touching-pair cubature at 1000 evaluations
    # (TaylorDuffy.cc:263-272): its entries carry ~1e-6 of the largest entry
    assert relerr(M, d["M"]) < 2e-6, relerr(M, d["M"])
    # FP32 far field: phases k r up to ~50 rad here keep ~50 * 2^-24 relative
    M32 = G.AssembleBEMMatrix(w, precision="mixed").numpy()
    assert np.abs(M32 - M).max() / np.abs(M).max() < 2e-5


def test_block_assembly_matches_full_matrix(golden):
    """AssembleBEMMatrixBlock: the four surface blocks of two PEC spheres at
    imaginary frequency, at offsets inside a larger array, equal the
    corresponding blocks of the full matrix; F64 blocks are its real part."""
    from gbem import RWGGeometry
    d = golden("ref_pec2_s1_xi.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    M = G.AssembleBEMMatrix(w).numpy()
    n0, n1 = G.NumBFs(0), G.NumBFs(1)
    off = [0, n0]
    assert n0 + n1 == M.shape[0]
    assert np.abs(M.imag).max() <= 1e-14 * np.abs(M).max()  # real at imaginary frequency
    for a in range(2):
        for b in range(2):
            ref = M[off[a]:off[a] + G.NumBFs(a), off[b]:off[b] + G.NumBFs(b)]
            big = np.zeros((G.NumBFs(a) + 5, G.NumBFs(b) + 3), dtype=np.complex128, order="F")
            G.AssembleBEMMatrixBlock(a, b, w, big, RowOffset=5, ColOffset=3)
            assert np.array_equal(big[5:, 3:], ref)
            assert not big[:5].any() and not big[:, :3].any()
            R = G.AssembleBEMMatrixBlock(a, b, w, real=True)
            assert R.dtype == np.float64 and np.array_equal(R, ref.real)


def test_f64_matrix_and_lu(golden):
    """Real (F64) storage at imaginary frequency: the assembled matrix is the
    real part of the C128 one and its LU matches LAPACK dgetrf's pivots."""
    import scipy.linalg as sl
    from gbem import RWGGeometry
    from gbem.api import HMatrix
    from gbem._lib import F64
    d = golden("ref_pec2_s1_xi.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    M = G.AssembleBEMMatrix(w).numpy()
    R = G.AssembleBEMMatrix(w, HMatrix(G, F64))
    A = R.numpy()
    assert A.dtype == np.float64 and np.array_equal(A, M.real)
    assert R.LUFactorize() == 0
    lu, piv = sl.lu_factor(A)
    assert np.array_equal(R.ipiv - 1, piv)
    assert np.abs(R.numpy() - lu).max() / np.abs(lu).max() < 1e-12
    b = np.random.default_rng(5).standard_normal((A.shape[0], 2))
    x = R.LUSolve(b)
    assert np.abs(A @ x - b).max() / np.abs(b).max() < 1e-10
