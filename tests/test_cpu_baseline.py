"""The CPU baseline's pieces (oracle/cpu_solve.py): the panel-by-panel LU
is zgetrf (same pivots, same factors), and the slices of one solve add up to
the whole solve."""
import numpy as np
import scipy.linalg as sl


def test_blocked_lu_is_zgetrf():
    from oracle.cpu_solve import BlockedLU
    N = 700
    rng = np.random.default_rng(1)
    A0 = np.asfortranarray(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N)))
    lu = BlockedLU(A0.copy(order="F"), nb=128)
    lu.panels(0, 2)
    lu.panels(2, lu.npanels)
    lu2, piv = sl.lu_factor(A0)
    assert np.array_equal(lu.ipiv - 1, piv)
    assert np.abs(lu.A - lu2).max() / np.abs(lu2).max() < 1e-12
    B = np.asfortranarray(rng.standard_normal((N, 3)) + 0j)
    X = B.copy(order="F")
    assert lu.solve(X) == 0
    assert np.abs(A0 @ X - B).max() / np.abs(B).max() < 1e-10
    assert abs(lu.total_flops() / (8.0 * N ** 3 / 3.0) - 1.0) < 1e-12


def test_slices_cover_one_solve():
    from oracle.cpu_solve import SlicedSolve
    job = SlicedSolve(subdiv=1, warm=True)
    eb = job.stripe_bounds(5)
    kb = job.panel_bounds(3)
    fa = sum(job.assemble(eb[j], eb[j + 1])[1] for j in range(5))
    fl = sum(job.factor(kb[j], kb[j + 1])[1] for j in range(3))
    assert abs(fa - 1.0) < 1e-12 and abs(fl - 1.0) < 1e-12
    from oracle import oracle
    M = oracle.assemble([job.S], [(0, 1)], [False], job.omega, job.eps, [1.0, 1.0])
    assert np.array_equal(np.triu(job.M), np.triu(M))
