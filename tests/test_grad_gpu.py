"""Gradients through the kernels on the GPU: the autograd matvec against torch's numerical
Jacobian, the local-energy gradient, and dE/dJ_i of the disordered XXZ chain by Hellmann-Feynman
against exact diagonalisation, the reference's own mpo_expectation of dH/dJ_i (tests/golden/
grad_xxz10.json) and central finite differences of DMRG energies (h = 1e-5, the bar 1e-6
relative)."""
import itertools

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


def _small(seed):
    from tnkit_gb300 import workloads
    return workloads.mid_bond_problem(dims=(1, 2, 3, 2, 1), charges=(-4, -2, 0, 2, 4), seed=seed)


def test_matvec_gradcheck():
    from tnkit_gb300.grad import TwoSiteMatvec
    th, L, W1, W2, R = _small(1)
    x = th.data.clone().requires_grad_(True)
    f = lambda t: TwoSiteMatvec.apply(t, th.layout, L, W1, W2, R)
    assert torch.autograd.gradcheck(f, (x,), eps=1e-6, atol=1e-9, rtol=1e-7)


def test_local_energy_gradient():
    from tnkit_gb300 import ops
    from tnkit_gb300.grad import local_energy
    th, L, W1, W2, R = _small(2)
    # random environments make H_eff non-symmetric: the exact gradient of x^T H x / x^T x is
    # ((H + H^T) x - 2 E x) / x^T x
    x = th.data.clone().requires_grad_(True)
    e = local_energy(x, th.layout, L, W1, W2, R)
    e.backward()
    op = ops.TwoSiteOperator(th.layout, L, W1, W2, R)
    from tnkit_gb300.grad import TwoSiteMatvec
    xd = th.data
    hx = op(xd)
    n2 = float(torch.dot(xd, xd))
    E = float(torch.dot(xd, hx)) / n2
    # gradient = (H x + H^T x) / n2 - 2 E x / n2; H^T x via the autograd backward of y = H x
    xx = xd.clone().requires_grad_(True)
    y = TwoSiteMatvec.apply(xx, th.layout, L, W1, W2, R)
    (htx_,) = torch.autograd.grad(y, xx, grad_outputs=xd)
    want = (hx + htx_) / n2 - 2 * E * xd / n2
    assert abs(float(e.detach()) - E) <= 1e-13 * abs(E)
    assert float((x.grad - want).abs().max()) <= 1e-12 * float(want.abs().max())


def _ed_bond_terms(J, delta):
    from tnkit_gb300 import workloads
    W = workloads.xxz_disordered_mpo(J, delta)
    T = W[0][0]
    for Wn in W[1:]:
        T = np.einsum("wab,wxcd->xacbd", T, Wn)
        T = T.reshape(T.shape[0], T.shape[1] * T.shape[2], -1)
    H = T[0]
    N = len(J) + 1
    idx = [i for i, ss in enumerate(itertools.product(range(2), repeat=N)) if sum(ss) == N // 2]
    ev, evec = np.linalg.eigh(H[np.ix_(idx, idx)])
    psi = np.zeros(2 ** N)
    psi[idx] = evec[:, 0]
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm, sz = sp.T.copy(), np.diag([0.5, -0.5])
    h = 0.5 * (np.kron(sp, sm) + np.kron(sm, sp)) + delta * np.kron(sz, sz)
    out = []
    for i in range(N - 1):
        t = psi.reshape(2 ** i, 4, -1)
        out.append(float(np.einsum("axb,xy,ayb->", t, h, t)))
    return float(ev[0]), np.array(out)


def _dmrg_xxz(J, delta, chi=32):
    from tnkit_gb300 import workloads
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.mpo import to_block_mpo
    N = len(J) + 1
    Wb, _ = to_block_mpo(workloads.xxz_disordered_mpo(J, delta), [[1, -1]] * N)
    return dmrg(Wb, chi, charge=0, seed=1, n_sweeps=8, tol=1e-14, rtol=0, expand=0,
                eig_tol=1e-12)


def test_hellmann_feynman_gradient_matches_exact_and_finite_differences():
    from tnkit_gb300.grad import energy_gradient_xxz
    N, delta = 10, 1.0
    J = np.random.default_rng(2).uniform(0.5, 1.5, N - 1)
    E, M, info = _dmrg_xxz(J, delta)
    E_ed, g_ed = _ed_bond_terms(J, delta)
    assert abs(E - E_ed) <= 1e-11 * abs(E_ed)
    g = energy_gradient_xxz(M, delta)
    assert np.abs(g - g_ed).max() <= 1e-8 * np.abs(g_ed).max(), (g, g_ed)
    assert abs(float(J @ g) - E) <= 1e-10 * abs(E)          # E = sum_i J_i <h_i>
    h = 1e-5                      # the central-difference step the configuration names
    for i in (0, 4, 8):
        Jp, Jm = J.copy(), J.copy()
        Jp[i] += h
        Jm[i] -= h
        fd = (_dmrg_xxz(Jp, delta)[0] - _dmrg_xxz(Jm, delta)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * abs(g[i]), (i, fd, g[i])


@pytest.mark.parametrize("model", ["xxz", "tfim"])
def test_mps_energy_gradient_finite_differences(model):
    """dE/dA_i of the Rayleigh quotient by environment recomputation against central finite
    differences of E (h = 1e-5) on entries of every site tensor of a random, non-canonical MPS,
    and E against the dense energy of the same state (dense H from the same MPO tensors, every
    leg in sector order)."""
    from tnkit_gb300 import workloads
    from tnkit_gb300.grad import mps_energy_gradient
    from tnkit_gb300.layout import to_dense_np
    from tnkit_gb300.mpo import dense_mpo, random_block_mps, random_dense_mps, to_block_mpo
    rng = np.random.default_rng(11)
    N = 6
    if model == "xxz":
        Wb = to_block_mpo(workloads.xxz_mpo(N, 0.7), [[1, -1]] * N)[0]
        M = random_block_mps(Wb, 6, 0, np.random.default_rng(3), device="cuda")
    else:
        Wb = dense_mpo(workloads.tfim_mpo(N, 0.8))
        M = random_dense_mps(N, 5, 2, np.random.default_rng(4), device="cuda")
    E, g = mps_energy_gradient(M, Wb)
    psi = np.ones((1, 1))
    for m in M:
        psi = np.tensordot(psi, to_dense_np(m.layout, m.data.cpu().numpy()), axes=(-1, 0))
    psi = psi.reshape(-1)
    H = None
    for w in Wb:
        Wd = to_dense_np(w.layout, w.data.cpu().numpy())
        if H is None:
            H = Wd
        else:
            a, c = H.shape[0], Wd.shape[1]
            H = np.einsum("abij,bckl->acikjl", H, Wd).reshape(
                a, c, H.shape[2] * Wd.shape[2], H.shape[3] * Wd.shape[3])
    H = H[0, 0]
    Eex = float(psi @ H @ psi / (psi @ psi))
    assert abs(E - Eex) <= 1e-12 * abs(Eex), (E, Eex)
    h = 1e-5
    for i, A in enumerate(M):
        for k in rng.choice(A.data.numel(), size=min(3, A.data.numel()), replace=False):
            k = int(k)
            x0 = float(A.data[k])
            A.data[k] = x0 + h
            Ep, _ = mps_energy_gradient(M, Wb)
            A.data[k] = x0 - h
            Em, _ = mps_energy_gradient(M, Wb)
            A.data[k] = x0
            fd = (Ep - Em) / (2 * h)
            assert abs(fd - float(g[i].data[k])) <= 1e-6 * max(1.0, abs(fd)), (i, k, fd)


def test_hellmann_feynman_gradient_matches_reference_mpo_expectation():
    """dE/dJ_i of the disordered XXZ chain (N=10, J from seed 2) against the reference's
    mpo_expectation(psi, dH/dJ_i) on its own complex128 ground state (tnkit/dmrg_excited.py:
    185-211), and the reference's central finite differences (h = 1e-5)."""
    import json
    import os
    from conftest import GOLDEN
    from tnkit_gb300.grad import energy_gradient_xxz
    ref = json.load(open(os.path.join(GOLDEN, "grad_xxz10.json")))
    J = np.asarray(ref["J"])
    E, M, info = _dmrg_xxz(J, ref["delta"], chi=ref["chi"])
    assert abs(E - ref["E"]) <= 1e-12 * abs(ref["E"])
    g = energy_gradient_xxz(M, ref["delta"])
    hf = np.asarray(ref["hf_grad"])
    assert np.abs(g - hf).max() <= 1e-8 * np.abs(hf).max(), (g, hf)
    for i, fd in ref["fd_grad"].items():
        assert abs(g[int(i)] - fd) <= 1e-6 * abs(fd)
