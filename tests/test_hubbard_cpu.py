"""U(1) x U(1) blocks (the Fermi-Hubbard chain's (N_up, N_dn) labels) on the host: the block MPO
and the seeded random block MPS are the reference's, element for element (golden vectors from
tests/golden/make_golden.py hubbard, made by running the reference's to_block_mpo and
random_block_mps under ProductSymmetry((U1(), U1()))); the hand-written MPO is the Jordan-Wigner
Hamiltonian."""
import itertools
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import GOLDEN


@pytest.fixture(scope="module")
def hub():
    meta = json.load(open(os.path.join(GOLDEN, "hubbard_u1u1.json")))
    arrays = dict(np.load(os.path.join(GOLDEN, "hubbard_u1u1.npz")))
    return meta, arrays


def _legs(t):
    return [{"charges": [list(c) for c in l.charges], "dims": list(l.dims), "sign": l.sign}
            for l in t.legs]


def test_block_mpo_matches_reference(hub):
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import to_block_mpo
    meta, arrays = hub
    Wb, _ = to_block_mpo(workloads.hubbard_mpo(6), [workloads.HUBBARD_SITE_CHARGES] * 6,
                         device="cpu")
    assert _legs(Wb[2]) == meta["mpo_site2"]["legs"]
    assert np.array_equal(Wb[2].data.numpy(), arrays["mpo_site2"])


def test_random_block_mps_matches_reference(hub):
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import random_block_mps, to_block_mpo
    meta, arrays = hub
    Wb, _ = to_block_mpo(workloads.hubbard_mpo(6), [workloads.HUBBARD_SITE_CHARGES] * 6,
                         device="cpu")
    M = random_block_mps(Wb, 16, (3, 3), np.random.default_rng(1), device="cpu")
    assert [_legs(m) for m in M] == [m["legs"] for m in meta["mps_seed1_chi16"]]
    for i in (0, 2):
        assert np.array_equal(M[i].data.numpy(), arrays[f"mps_seed1_chi16_site{i}"])


def test_hubbard_mpo_is_the_jordan_wigner_hamiltonian(hub):
    """The dense MPO of N=3 equals the Hamiltonian built from 2N Jordan-Wigner fermion modes,
    and the N=6 half-filled ground energy is the fixture's exact value."""
    from tnkit_gb300 import workloads
    meta, _ = hub

    def dense(W):
        T = W[0][0]
        for Wn in W[1:]:
            T = np.einsum("wab,wxcd->xacbd", T, Wn)
            T = T.reshape(T.shape[0], T.shape[1] * T.shape[2], -1)
        return T[0]

    N, t, U = 3, 1.0, 4.0
    a = np.array([[0.0, 1.0], [0.0, 0.0]])
    Z, I2 = np.diag([1.0, -1.0]), np.eye(2)

    def mode(k):
        out = np.ones((1, 1))
        for m in [Z] * k + [a] + [I2] * (2 * N - k - 1):
            out = np.kron(out, m)
        return out
    c = [mode(k) for k in range(2 * N)]
    H = np.zeros((4 ** N, 4 ** N))
    for j in range(N - 1):
        for s in range(2):
            p, q = 2 * j + s, 2 * j + 2 + s
            H -= t * (c[p].T @ c[q] + c[q].T @ c[p])
    for j in range(N):
        H += U * (c[2 * j].T @ c[2 * j]) @ (c[2 * j + 1].T @ c[2 * j + 1])
    # site state s = |0>,|up>,|dn>,|up dn> is mode occupation (n_up, n_dn) -> index 2 n_up + n_dn
    occ = [0, 2, 1, 3]
    perm = [sum(occ[s] * 4 ** (N - 1 - i) for i, s in enumerate(ss))
            for ss in itertools.product(range(4), repeat=N)]
    Hm = dense(workloads.hubbard_mpo(N, t, U))
    assert np.abs(Hm - H[np.ix_(perm, perm)]).max() == 0.0
    H6 = dense(workloads.hubbard_mpo(6, t, U))
    q = np.array(workloads.HUBBARD_SITE_CHARGES)
    idx = [i for i, ss in enumerate(itertools.product(range(4), repeat=6))
           if tuple(q[list(ss)].sum(0)) == (3, 3)]
    assert abs(np.linalg.eigvalsh(H6[np.ix_(idx, idx)])[0] - meta["n6_exact_E"]) <= 1e-12
