"""Host logic of the autograd shape derivative (gbem.adjoint) on a toy
problem with the same structure -- a complex-symmetric M(V) and b(V), both
affine in the vertex coordinates -- whose contractions are written out in
numpy: the adjoint solve, the signs of the two contractions and PyTorch's
complex-gradient convention against central differences."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


class _FakeMatrix:
    def __init__(self, M):
        self.M = M

    def LUFactorize(self):
        return 0

    def LUSolve(self, B):
        return np.linalg.solve(self.M, B)


class _FakeGeometry:
    def __init__(self, theta, A0, A, b0, Bk, waves):
        self.theta, self.A0, self.A, self.b0, self.Bk, self.waves = theta, A0, A, b0, Bk, waves

    def _M(self):
        return self.A0 + np.tensordot(self.theta, self.A, axes=1)

    def AssembleBEMMatrix(self, Omega):
        return _FakeMatrix(self._M())

    def AssembleRHSVector(self, Omega, E0, nh):
        w = [tuple(e) for e, _ in self.waves].index(tuple(E0))
        return self.b0[:, w] + np.tensordot(self.theta, self.Bk[:, :, w], axes=1)

    def solve_mixed(self, Omega, B):
        return np.linalg.solve(self._M(), B), 1, 0.0

    def VertexVJP(self, Omega, lam, x, rel_step=1e-4):
        g = np.array([np.real(np.sum(np.conj(lam) * (Ak @ x))) for Ak in self.A])
        return g.reshape(-1, 3)

    def RHSVertexVJP(self, Omega, waves, gb):
        return np.real(np.einsum("iw,kiw->k", np.conj(gb), self.Bk)).reshape(-1, 3)

    def basis_types(self):
        return np.array([0, 1] * (self.A0.shape[0] // 2), dtype=np.int8)


class _FakeTopology:
    def __init__(self, nv, N, nw, seed=0):
        rng = np.random.default_rng(seed)
        K = 3 * nv

        def sym(*shape):
            a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
            return a + np.swapaxes(a, -1, -2)
        self.A0 = sym(N, N) + 8 * np.eye(N)
        self.A = 0.3 * sym(K, N, N)
        self.b0 = rng.standard_normal((N, nw)) + 1j * rng.standard_normal((N, nw))
        self.Bk = 0.3 * (rng.standard_normal((K, N, nw)) + 1j * rng.standard_normal((K, N, nw)))
        self.waves = [((1.0 + w, 0.0, 0.0), (0.0, 0.0, 1.0)) for w in range(nw)]
        self.num_vertices = nv

    def geometry(self, V):
        return _FakeGeometry(np.asarray(V).ravel(), self.A0, self.A, self.b0, self.Bk, self.waves)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autograd_gradient_of_extinction_matches_central_differences(precision):
    from gbem.adjoint import extinction_power, scatter
    topo = _FakeTopology(nv=3, N=6, nw=2)
    V0 = np.random.default_rng(1).standard_normal((3, 3)) * 0.1

    def power(V, grad):
        Vt = torch.tensor(V, requires_grad=grad)
        x, b = scatter(Vt, topo, 1.0, topo.waves, precision=precision)
        p = extinction_power(x, b, topo.geometry(V).basis_types()).sum()
        if grad:
            p.backward()
            return Vt.grad.numpy()
        return float(p)

    g = power(V0, True)
    h = 1e-6
    fd = np.zeros_like(V0)
    for q in range(V0.size):
        Vp, Vm = V0.copy(), V0.copy()
        Vp.flat[q] += h
        Vm.flat[q] -= h
        fd.flat[q] = (power(Vp, False) - power(Vm, False)) / (2 * h)
    assert np.abs(fd - g).max() / np.abs(g).max() < 1e-7
