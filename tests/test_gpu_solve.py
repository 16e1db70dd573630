"""Right-hand sides and the mixed-precision solve."""
import numpy as np
import pytest

from helpers import fixture_surfaces, omega_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,j", [("pec_s2_w1", 0), ("diel_s1_w2", 0), ("diel_s1_w2", 1)])
def test_planewave_rhs_matches_reference(golden, case, j):
    from gbem import RWGGeometry
    d = golden("ref_%s.npz" % case)
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    pw = d["pw%d" % j]
    b = G.AssembleRHSVector(omega_of(d), pw[:3], pw[3:])
    ref = d["rhs%d" % j]
    assert np.abs(b - ref).max() / np.abs(ref).max() < 1e-12


def test_mixed_solve_refines_to_fp64(golden):
    import scipy.linalg as sl
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(2)
    G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}])
    w = 2.0
    B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in
                  [((1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1)), ((1, 0, 0), (0, 0, -1)), ((0, 1, 0), (0, 0, -1))]],
                 axis=1)
    X, it, res = G.solve_mixed(w, B, tol=1e-10, max_iter=12)
    assert res <= 1e-10 and 1 <= it <= 12
    # the refined solution solves the mixed-assembled (complex64) matrix to FP64 accuracy
    M32 = G.AssembleBEMMatrix(w, precision="mixed").numpy().astype(np.complex128)
    assert np.abs(M32 @ X - B).max() / np.abs(B).max() < 1e-9
    # and differs from the FP64 path only by the complex64 storage of the
    # matrix (the far field is float-float, ~1e-11 per entry before rounding)
    M64 = G.AssembleBEMMatrix(w).numpy()
    assert np.abs(M32 - M64).max() / np.abs(M64).max() < 1e-7
    X64 = sl.solve(M64, B)
    assert np.abs(X - X64).max() / np.abs(X64).max() < 1e-5


@pytest.mark.parametrize("case", ["pec_s2_w1", "diel_s1_w2"])
def test_emt_power_matches_reference(golden, case):
    """Scattered and absorbed power (EMT, GetPFT) of the reference's own
    solutions: the GPU quadratic form with the exterior-region matrix agrees
    with the reference and with the oracle's restatement."""
    from gbem import RWGGeometry
    from oracle import oracle as ora
    d = golden("ref_%s.npz" % case)
    gs, (regs, pec, eps, mu) = fixture_surfaces(d)
    G = RWGGeometry(gs)
    w = omega_of(d)
    j = 0
    while "kn%d" % j in d.files:
        kn, rhs, ref = d["kn%d" % j], d["rhs%d" % j], d["pft%d" % j]
        pabs, pscat = G.GetPFT(w, kn, RHS=rhs)
        po = ora.emt_pscat(ora.Surface(gs[0]["V"], gs[0]["P"]), pec[0], w, kn)
        assert abs(pscat[0] - po) < 1e-9 * abs(po), (pscat, po)
        assert abs(pscat[0] - ref[1]) < 2e-6 * abs(ref[1]), (pscat, ref)
        # absorbed = extinction - scattered (zero up to quadrature for PEC)
        assert abs(pabs[0] - ref[0]) < 2e-6 * abs(ref[1]), (pabs, ref)
        _, p32 = G.GetPFT(w, kn, precision="mixed")
        assert abs(p32[0] - pscat[0]) < 1e-6 * abs(pscat[0])
        j += 1


def _sphere_powers(G, w, B, precision):
    if precision == "mixed":
        X, _, _ = G.solve_mixed(w, B)
    else:
        M = G.AssembleBEMMatrix(w)
        M.LUFactorize()
        X = M.LUSolve(B.copy())
    return G.GetPFT(w, X, RHS=B)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sphere_powers_against_mie(precision):
    """Scattered and absorbed power of icosphere meshes against the Mie series
    (oracle/mie.py): the PEC sphere of the plain small workload (s = 2, kR = 1,
    x-polarised wave along +z) and the eps = 2.25+0.01i sphere at kR = 2 on
    s = 2 and s = 3 meshes.  The difference is the mesh's (flat panels): it
    falls about fourfold per subdivision (measured 3.8e-2 PEC s=2; 2.9e-2 /
    4.6e-2 and 7.2e-3 / 1.2e-2 absorbed / scattered for the dielectric at
    s = 2, 3)."""
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    from oracle import mie
    pw = [((1, 0, 0), (0, 0, 1))]
    V, P = mesh.icosphere(2)
    G = RWGGeometry([{"V": V, "P": P}])
    B = np.stack([G.AssembleRHSVector(1.0, e, n) for e, n in pw], axis=1)
    pa, ps = _sphere_powers(G, 1.0, B, precision)
    _, ms = mie.powers(1.0, pec=True)
    assert abs(ps[0] - ms) < 5e-2 * ms and abs(pa[0]) < 1e-8 * ms
    errs = []
    for s in (2, 3):
        V, P = mesh.icosphere(s)
        G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}])
        B = np.stack([G.AssembleRHSVector(2.0, e, n) for e, n in pw], axis=1)
        pa, ps = _sphere_powers(G, 2.0, B, precision)
        ma, ms = mie.powers(2.0, eps=2.25 + 0.01j)
        errs.append((abs(pa[0] - ma) / ma, abs(ps[0] - ms) / ms))
    assert errs[0][0] < 5e-2 and errs[0][1] < 7e-2
    assert errs[1][0] < 1.5e-2 and errs[1][1] < 2e-2
    assert errs[1][0] < 0.5 * errs[0][0] and errs[1][1] < 0.5 * errs[0][1]


def test_batch_matches_individual_solves():
    """gbem_solve_mixed_batch: concurrent jobs on different geometries (and
    frequency sweeps on one geometry, serialised on it) give the results of
    the one-at-a-time solves."""
    from gbem import RWGGeometry, mesh, solve_mixed_batch
    from gbem.api import Material
    pw = [((1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, -1))]
    geos = []
    for s, mat in ((1, Material(2.25 + 0.01j)), (2, Material(4.0 + 0.1j)), (1, None)):
        V, P = mesh.icosphere(s)
        geos.append(RWGGeometry([{"V": V, "P": P, "material": mat}]))
    jobs = []
    for G in geos:
        for w in (0.5, 2.0):
            jobs.append((G, w, np.stack([G.AssembleRHSVector(w, e, n) for e, n in pw], axis=1)))
    ref = [G.solve_mixed(w, B)[0] for G, w, B in jobs]
    out = solve_mixed_batch(jobs, max_concurrent=3)
    for (X, it, res), Xr in zip(out, ref):
        assert res <= 1e-10 and it >= 1
        assert np.abs(X - Xr).max() <= 1e-12 * np.abs(Xr).max()


def test_refined_solve_is_the_fp64_solve():
    """gbem_solve_refined: FP64 matrix, tensor-core LU of its complex64
    rounding, FP64 residuals against the FP64 matrix -- the FP64 solve's
    solution to the refinement tolerance."""
    import scipy.linalg as sl
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(2)
    G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}])
    w = 2.0
    B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in [((1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, -1))]], axis=1)
    X, it, res = G.solve_refined(w, B, tol=1e-13)
    assert res <= 1e-13
    M64 = G.AssembleBEMMatrix(w).numpy()
    X64 = sl.solve(M64, B)
    assert np.abs(X - X64).max() / np.abs(X64).max() < 1e-11


def test_gmres_refinement_on_an_ill_conditioned_matrix():
    """At low frequency the PMCHWT matrix of a fine jittered mesh is
    ill-conditioned enough that plain refinement with the complex64 factor
    diverges (the batching workload's second geometry, a seeded rounded cube
    of 2700 panels, N = 8100, at kR = 0.1); the solve switches to GMRES-based
    refinement preconditioned by the same factor and reaches the tolerance,
    against the FP64 solution."""
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    rng = np.random.default_rng(0)  # the batching workload's draws, seed 0
    rng.uniform(1.5, 4.0), rng.uniform(0.0, 0.1), rng.uniform(0.5, 1.5)
    eps = complex(rng.uniform(1.5, 4.0), rng.uniform(0.0, 0.1))
    npan = int(rng.uniform(600, 3000))
    V, P = mesh.rounded_cube(npan, side=1.0, seed=int(rng.integers(1 << 30)))
    G = RWGGeometry([{"V": V, "P": P, "material": Material(eps)}])
    w = 0.1 / 0.5
    B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in [((1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1))]], axis=1)
    X, it, res = G.solve_mixed(w, B, tol=1e-10, max_iter=12)
    print("rounded cube N=%d kR=0.1: mixed sweeps %d, residual %.2e" % (G.TotalBFs, it, res))
    assert res <= 1e-10
    # the mixed form solves its complex64 matrix: the refinement residual is
    # taken against it (rounding the matrix moves this ill-conditioned
    # solution by ~1e-3, so it is not compared with the FP64 solution); the
    # sweeps stop at a 2-norm relative residual of 1e-10, so the largest entry
    # of the residual may exceed 1e-10 of the largest entry of B by ~sqrt(N)
    M32 = G.AssembleBEMMatrix(w, precision="mixed").numpy().astype(np.complex128)
    assert np.abs(M32 @ X - B).max() / np.abs(B).max() < 1e-8
    # the refined form keeps the FP64 matrix and reaches the FP64 solution
    Xr, itr, resr = G.solve_refined(w, B, tol=1e-12, max_iter=12)
    print("refined sweeps %d, residual %.2e" % (itr, resr))
    assert resr <= 1e-12
    # two FP64-accurate solutions of a matrix this ill-conditioned differ by
    # ~cond x 1e-16 (measured 1.4e-8 between them)
    M = G.AssembleBEMMatrix(w)
    assert M.LUFactorize() == 0
    X64 = M.LUSolve(B)
    assert np.abs(Xr - X64).max() / np.abs(X64).max() < 1e-7


def _bipyramid(center, r=0.3, h=0.4):
    """Closed triangular bipyramid (6 outward-oriented panels, 9 edges): an
    odd number of RWG functions for a PEC body."""
    c = np.asarray(center, dtype=np.float64)
    eq = [c + r * np.array([np.cos(a), np.sin(a), 0.0]) for a in (0.0, 2 * np.pi / 3, 4 * np.pi / 3)]
    V = np.array([c + [0, 0, h], c - [0, 0, h]] + eq)
    P = np.array([[0, 2, 3], [0, 3, 4], [0, 4, 2], [1, 3, 2], [1, 4, 3], [1, 2, 4]], dtype=np.int32)
    return V, P


def test_mixed_solve_with_odd_n():
    """An odd number of basis functions (a PEC sphere and a PEC bipyramid,
    N = 1920 + 9 = 1929): partial leaves, tile edges and the last triangular
    block of the complex-FP32 path; the refined solution equals the FP64 one."""
    import scipy.linalg as sl
    from gbem import RWGGeometry, mesh
    V, P = mesh.icosphere(3)
    Vb, Pb = _bipyramid((2.2, 0.0, 0.0))
    G = RWGGeometry([{"V": V, "P": P, "material": None}, {"V": Vb, "P": Pb, "material": None}])
    assert G.TotalBFs % 2 == 1
    w = 1.0
    B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in [((1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1))]],
                 axis=1)
    X, it, res = G.solve_mixed(w, B, tol=1e-10, max_iter=12)
    assert res <= 1e-10
    X64 = sl.solve(G.AssembleBEMMatrix(w).numpy(), B)
    assert np.abs(X - X64).max() / np.abs(X64).max() < 1e-5
