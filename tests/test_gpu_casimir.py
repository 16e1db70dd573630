"""The scuff-cas3D integrand on the GPU: two PEC icospheres (subdivision 3,
1280 panels and 1920 RWG edges each, N = 3840 real), centres 3 apart, at the
20-point Gauss-Laguerre frequencies xi = x_j / g for g = 1 (surface gap) and
g = 3 (centre gap).

* The energy and z-force integrands against the reference's own (its
  unchanged scuff-cas3D, GetCasimirIntegrand, CasimirIntegrand.cc:243-480,
  run by tests/golden/make_golden.py on the same mesh).
* The U block and its derivative dU/dz against the oracle (assembly, and
  central differences of the assembly) at one frequency."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bodies():
    from gbem import mesh
    V, P = mesh.icosphere(3)
    return V, P, [{"V": V, "P": P, "material": None}, {"V": V + [0.0, 0.0, 3.0], "P": P, "material": None}]


@pytest.fixture(scope="module")
def cas():
    from gbem.casimir import CasimirIntegrand
    return CasimirIntegrand(_bodies()[2])


def test_casimir_integrand_matches_reference(cas, golden):
    d = golden("ref_pec2_s3_casimir.npz")
    E = np.zeros(len(d["xi"]))
    F = np.zeros(len(d["xi"]))
    for i, xi in enumerate(d["xi"]):
        E[i], F[i] = cas(float(xi))
    for g in (1.0, 3.0):
        sel = d["gap"] == g
        # scale: the largest integrand over the rule (the integrands fall off
        # by e^{-2 xi gap}); the reference's adaptive near-field cubature
        # carries ~1e-6 relative of each T block's entries
        eE = np.abs(E[sel] - d["energy"][sel]).max() / np.abs(d["energy"][sel]).max()
        eF = np.abs(F[sel] - d["zforce"][sel]).max() / np.abs(d["zforce"][sel]).max()
        print("gap %g: energy %.2e force %.2e" % (g, eE, eF))
        assert eE < 1e-5, (g, eE)
        assert eF < 1e-5, (g, eF)


def test_u_block_and_gradient_match_oracle(cas, golden):
    from oracle import oracle
    V, P, bodies = _bodies()
    G = cas.G
    xi = float(golden("ref_pec2_s3_casimir.npz")["xi"][9])
    n1 = G.NumBFs(0)
    U = G.AssembleBEMMatrixBlock(0, 1, 1j * xi, real=True)
    dUz = G.AssembleBEMMatrixBlockGradient(0, 1, 1j * xi, real=True, components=(2,))[2]
    rng = np.random.default_rng(4)
    cols = np.sort(rng.choice(n1, 12, replace=False))

    def ora_u(dz):
        Sa = oracle.Surface(V + [0.0, 0.0, dz], P)
        Sb = oracle.Surface(V + [0.0, 0.0, 3.0], P)
        M = oracle.assemble_cols([Sa, Sb], [(0, -1), (0, -1)], [True, True], 1j * xi, [1.0], [1.0], n1 + cols)
        return M[:n1]

    Uo = ora_u(0.0)
    assert np.abs(Uo.imag).max() <= 1e-14 * np.abs(Uo).max()
    assert np.abs(U[:, cols] - Uo.real).max() / np.abs(Uo).max() < 1e-11
    h = 1e-4
    dUo = (ora_u(h) - ora_u(-h)).real / (2 * h)
    # central differences: truncation ~h^2 of the entries' third derivative
    assert np.abs(dUz[:, cols] - dUo).max() / np.abs(dUo).max() < 1e-6
