"""Gradient of a time-evolved observable through two-site TDVP on the GPU
(grad.tdvp_observable_gradient: forward TDVP of psi, backward TDVP of Z psi(t), the integrand
Im <lam|h_i|psi> by polarisation over MPS sums on the matvec and environment kernels): on the
disordered XXZ chain N=8 from a full-rank random block state at full bond dimension, where
TDVP2 is exact, against exact diagonalisation (the Frechet derivative of exp(-iHt)) and
against central differences (h = 1e-5) of tdvp2_evolve itself."""
import numpy as np
import pytest
import scipy.linalg as sl

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

N, DELTA, DT, STEPS, SITE, CHI = 8, 1.0, 0.05, 20, 4, 16


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


def _mpo(J):
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import to_block_mpo
    return to_block_mpo(workloads.xxz_disordered_mpo(J, DELTA), [[1, -1]] * N)[0]


def _dense_H(W):
    """The MPO contracted to a matrix, physical legs in sector order (dense_vector's basis)."""
    T = W[0].to_dense()[0]                          # (wr, out, in)
    for w in W[1:]:
        d = w.to_dense()                            # (wl, wr, out, in)
        T = np.einsum("aOI,abij->bOiIj", T, d)
        T = T.reshape(T.shape[0], T.shape[1] * T.shape[2], T.shape[3] * T.shape[4])
    return T[0]


def _z_dense(site):
    # sector order of a site: charge -1 (2 S^z = -1) first, then +1
    z = np.array([-1.0, 1.0])
    return np.kron(np.kron(np.ones(2 ** site), z), np.ones(2 ** (N - site - 1)))


@pytest.fixture(scope="module")
def problem():
    from tnkit_gb300.grad import xxz_bond_operator
    from tnkit_gb300.mpo import random_block_mps, to_block_mpo
    J = np.random.default_rng(2).uniform(0.5, 1.5, N - 1)
    W = _mpo(J)
    B = to_block_mpo(xxz_bond_operator(DELTA), [[1, -1]] * 2)[0]
    mps0 = random_block_mps(W, CHI, 0, np.random.default_rng(5))
    return J, W, B, mps0


@pytest.fixture(scope="module")
def result(problem):
    from tnkit_gb300.grad import tdvp_observable_gradient
    J, W, B, mps0 = problem
    return tdvp_observable_gradient(mps0, W, B, CHI, DT, STEPS, SITE)


def test_tdvp_gradient_matches_exact_diagonalisation(problem, result):
    from tnkit_gb300.tdvp import dense_vector
    J, W, B, mps0 = problem
    value, g, info = result
    v0 = dense_vector(mps0)
    v0 = v0 / np.linalg.norm(v0)
    H = _dense_H(W)
    t = DT * STEPS
    A = -1j * H * t
    vt = sl.expm(A) @ v0
    Z = _z_dense(SITE)
    assert abs(value - np.vdot(vt, Z * vt).real) <= 1e-10
    exact = []
    for i in range(N - 1):
        e = np.zeros(N - 1)
        e[i] = 1.0
        h = _dense_H(_mpo(J + e)) - H               # dH/dJ_i (H is linear in J)
        dv = sl.expm_frechet(A, -1j * t * h, compute_expm=False) @ v0
        exact.append(2 * np.vdot(vt, Z * dv).real)
    exact = np.array(exact)
    assert info["points"] == STEPS + 1
    assert np.abs(g - exact).max() <= 1e-8 * np.abs(exact).max()


def test_tdvp_gradient_matches_central_differences(problem, result):
    from tnkit_gb300.tdvp import dense_vector, tdvp2_evolve
    J, W, B, mps0 = problem
    value, g, info = result
    h = 1e-5
    Z = _z_dense(SITE)

    def z_of(Jv):
        out, _ = tdvp2_evolve(list(mps0), _mpo(Jv), CHI, DT, STEPS)
        v = dense_vector(out)
        return float(np.vdot(v, Z * v).real / np.vdot(v, v).real)
    assert abs(z_of(J) - value) <= 1e-10
    for i in (1, SITE - 1, N - 2):
        e = np.zeros(N - 1)
        e[i] = h
        fd = (z_of(J + e) - z_of(J - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * np.abs(g).max()
