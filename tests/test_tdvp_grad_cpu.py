"""Host-side checks of the time-evolved observable gradient (tnkit_gb300.grad): the composite
Newton-Cotes weights, and the continuous-adjoint formula it integrates,
    d<Z(t)>/dJ_i = 2 int_0^t Im <lam(s)| h_i |psi(s)> ds,  lam(s) = exp(iH(t-s)) Z psi(t),
on a dense XXZ chain against the exact Frechet derivative of exp(-iHt) -- at the step the
TDVP gradient samples it (dt = 0.05, 20 steps)."""
import numpy as np
import pytest
import scipy.linalg as sl

from tnkit_gb300.grad import quadrature_weights


@pytest.mark.parametrize("n,deg", [(1, 1), (2, 3), (3, 3), (4, 5), (5, 3), (6, 3), (8, 5),
                                   (20, 5), (21, 3)])
def test_quadrature_weights_integrate_polynomials_exactly(n, deg):
    dt = 0.37
    s = np.arange(n + 1) * dt
    w = quadrature_weights(n, dt)
    for p in range(deg + 1):
        exact = (n * dt) ** (p + 1) / (p + 1)
        assert abs(w @ s ** p - exact) <= 1e-12 * max(1.0, exact)


def test_quadrature_weights_reject_empty_interval():
    with pytest.raises(ValueError):
        quadrature_weights(0, 0.1)


def _xxz_terms(N, delta):
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm, sz, one = sp.T.copy(), np.diag([0.5, -0.5]), np.eye(2)

    def op(o, i):
        m = np.array([[1.0]])
        for k in range(N):
            m = np.kron(m, o if k == i else one)
        return m
    return [0.5 * (op(sp, i) @ op(sm, i + 1) + op(sm, i) @ op(sp, i + 1))
            + delta * op(sz, i) @ op(sz, i + 1) for i in range(N - 1)], op


def test_continuous_adjoint_matches_exact_derivative():
    N, delta, dt, n, site = 6, 1.0, 0.05, 20, 3
    rng = np.random.default_rng(2)
    J = rng.uniform(0.5, 1.5, N - 1)
    h, op = _xxz_terms(N, delta)
    H = sum(j * hh for j, hh in zip(J, h))
    Z = 2 * op(np.diag([0.5, -0.5]), site)
    psi0 = rng.standard_normal(2 ** N) + 1j * rng.standard_normal(2 ** N)
    psi0 /= np.linalg.norm(psi0)
    t = n * dt
    A = -1j * H * t
    psi_t = sl.expm(A) @ psi0
    exact = np.array([2 * np.vdot(psi_t, Z @ (sl.expm_frechet(A, -1j * t * hh,
                                                             compute_expm=False) @ psi0)).real
                      for hh in h])
    step = sl.expm(-1j * H * dt)
    back = sl.expm(1j * H * dt)
    psi = [psi0]
    for _ in range(n):
        psi.append(step @ psi[-1])
    lam = [None] * (n + 1)
    lam[n] = Z @ psi[n]
    for k in range(n - 1, -1, -1):
        lam[k] = back @ lam[k + 1]
    g = np.array([[np.vdot(lam[k], hh @ psi[k]).imag for k in range(n + 1)] for hh in h])
    adj = 2 * g @ quadrature_weights(n, dt)
    assert np.abs(adj - exact).max() <= 1e-8 * np.abs(exact).max()
    # the polarisation identity the GPU path evaluates Im <lam|h|psi> with
    for k in (0, n // 2, n):
        for hh in h[:2]:
            m = lam[k] - 1j * psi[k]
            p = lam[k] + 1j * psi[k]
            pol = (np.vdot(m, hh @ m).real - np.vdot(p, hh @ p).real) / 4
            assert abs(pol - np.vdot(lam[k], hh @ psi[k]).imag) <= 1e-13


def _block_chain(N, chi, seed, cplx=True):
    import torch
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import random_block_mps, to_block_mpo
    W = to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N, device="cpu")[0]
    rng = np.random.default_rng(seed)
    mps = random_block_mps(W, chi, 0, rng, device="cpu")
    if cplx:
        from tnkit_gb300.tensor import BlockTensor
        mps = [BlockTensor(m.layout, m.data.to(torch.complex128)
                           * complex(*rng.standard_normal(2))) for m in mps]
    return W, mps


@pytest.mark.parametrize("N,chi_a,chi_b", [(2, 2, 2), (6, 8, 3), (8, 5, 16)])
def test_mps_sum_is_the_sum_of_the_states(N, chi_a, chi_b):
    """mps_sum's block copies (host-side layout logic; torch on the CPU here) give the dense
    vector |a> + c |b>, for bonds of different sectors and dims."""
    from tnkit_gb300.grad import mps_sum
    from tnkit_gb300.tdvp import dense_vector
    _, a = _block_chain(N, chi_a, 1)
    _, b = _block_chain(N, chi_b, 2)
    for c in (1.0, -1j, 0.3 + 2j):
        s = mps_sum(a, b, c)
        ref = dense_vector(a) + c * dense_vector(b)
        assert np.abs(dense_vector(s) - ref).max() <= 1e-13 * np.abs(ref).max()
        for m, x, y in zip(s[:-1], a[:-1], b[:-1]):
            assert m.legs[2].size == x.legs[2].size + y.legs[2].size


def test_apply_pauli_z_flips_the_down_components():
    from tnkit_gb300.grad import apply_pauli_z
    from tnkit_gb300.tdvp import dense_vector
    N, site = 6, 2
    _, a = _block_chain(N, 8, 3)
    z = np.array([-1.0, 1.0])                       # sector order: charge -1, then +1
    Z = np.kron(np.kron(np.ones(2 ** site), z), np.ones(2 ** (N - site - 1)))
    v = dense_vector(a)
    assert np.abs(dense_vector(apply_pauli_z(a, site)) - Z * v).max() <= 1e-14 * np.abs(v).max()
    assert np.abs(dense_vector(a) - v).max() == 0.0           # the input is not modified


def test_product_block_mps_is_the_neel_basis_state():
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import product_block_mps, to_block_mpo
    from tnkit_gb300.tdvp import dense_vector
    N = 6
    W = to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N, device="cpu")[0]
    neel = [1 if n % 2 == 0 else -1 for n in range(N)]
    v = dense_vector(product_block_mps(W, neel, device="cpu"))
    # sector order per site: charge -1 is index 0, charge +1 index 1
    k = sum((1 if s > 0 else 0) << (N - 1 - n) for n, s in enumerate(neel))
    ref = np.zeros(2 ** N)
    ref[k] = 1.0
    assert np.array_equal(v, ref)
    with pytest.raises(ValueError):
        product_block_mps(W, [2] + neel[1:], device="cpu")


def test_auxiliary_mpos_are_shared_and_correct():
    """The identity and Z MPOs the gradient contracts with are built once per chain and site
    (plans are cached by MPO object) and hold the right operators."""
    from tnkit_gb300.grad import _aux_mpo
    W, _ = _block_chain(4, 4, 1, cplx=False)
    assert _aux_mpo("id", W) is _aux_mpo("id", W)
    assert _aux_mpo("z", W, 1) is _aux_mpo("z", W, 1)
    assert _aux_mpo("z", W, 1) is not _aux_mpo("z", W, 2)
    for n, (i, z) in enumerate(zip(_aux_mpo("id", W), _aux_mpo("z", W, 1))):
        assert np.array_equal(i.to_dense()[0, 0], np.eye(2))
        # sector order: charge -1, then +1; Z = 2 S^z
        assert np.array_equal(z.to_dense()[0, 0], np.diag([-1.0, 1.0]) if n == 1 else np.eye(2))
