"""Pin the CPU oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py). CPU only."""
import json
import os

import numpy as np
import pytest

from oracle.blocks_np import BT, Leg, fuse, truncated_svd
from oracle import dmrg_np as O

from conftest import GOLDEN


def _bt(meta, arrays, key):
    return BT.from_json(meta[key], arrays[key])


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_block_two_site_matvec_matches_reference(golden, tag):
    meta, A = golden
    L, R, W1, W2, th = (_bt(meta, A, f"{tag}_{k}") for k in ("L", "R", "W1", "W2", "theta"))
    got = O.apply_two_site(th, L, W1, W2, R)
    ref = _bt(meta, A, f"{tag}_H2theta")
    assert [l for l in got.legs] == [l for l in ref.legs]
    assert _rel(got.flat(), ref.flat()) <= 1e-13


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_block_one_site_and_envs_match_reference(golden, tag):
    meta, A = golden
    L, W1, W2, R, R1 = (_bt(meta, A, f"{tag}_{k}") for k in ("L", "W1", "W2", "R", "R1"))
    Am, Bm = _bt(meta, A, f"{tag}_A"), _bt(meta, A, f"{tag}_B")
    assert _rel(O.apply_one_site(Am, L, W1, R1).flat(), A[f"{tag}_H1A"]) <= 1e-13
    assert _rel(O.update_left_env(L, Am, W1).flat(), A[f"{tag}_Lnext"]) <= 1e-13
    assert _rel(O.update_right_env(R, Bm, W2).flat(), A[f"{tag}_Rnext"]) <= 1e-13


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
@pytest.mark.parametrize("chi", [4, 10 ** 6])
def test_block_truncated_svd_matches_reference(golden, tag, chi):
    meta, A = golden
    mat = _bt(meta, A, f"{tag}_svdin")
    U, S, Vh, disc = truncated_svd(mat, chi)
    ref = meta[f"{tag}_S_chi{chi}"]
    assert np.allclose(S, A[f"{tag}_S_chi{chi}"], rtol=1e-12, atol=1e-14)
    assert abs(disc - ref["disc"]) <= 1e-12 * max(1.0, abs(ref["disc"]))
    bond = ref["bond"]
    assert list(U.legs[1].charges) == bond["charges"] and list(U.legs[1].dims) == bond["dims"]
    # the factors reproduce the matrix when nothing is cut
    if chi > mat.size:
        rec = np.zeros_like(mat.to_dense())
        ud, vd = U.to_dense(), Vh.to_dense()
        rec = (ud * S) @ vd
        assert _rel(rec, mat.to_dense()) <= 1e-12


def test_dense_two_site_matches_reference(golden):
    _, A = golden
    args = [A[f"tfim10_b4_{k}"] for k in ("theta", "L", "W1", "W2", "R")]
    ref = A["tfim10_b4_H2theta"]
    assert _rel(O.apply_two_site(*args), ref) <= 1e-13
    th, L, W1, W2, R = args
    assert _rel(O.apply_two_site_fused(th, *O.fused_two_site(L, W1, W2, R)), ref) <= 1e-12
    assert _rel(O.update_left_env(L, A["tfim10_b4_A"], W1), A["tfim10_b4_Lnext"]) <= 1e-13
    assert _rel(O.update_right_env(R, A["tfim10_b4_B"], W2), A["tfim10_b4_Rnext"]) <= 1e-13


def test_lanczos_restart_matches_reference(golden):
    meta, A = golden
    m = meta["lanczos"]
    H = A["lanczos_H"]
    e, x, info = O.lanczos_ground_restart(lambda v: H @ v, A["lanczos_v0"], tol=m["tol"],
                                          max_iter=m["max_iter"], m=m["m"], k=m["k"])
    assert abs(e - m["e"]) <= 1e-12 * abs(m["e"])
    assert info["iters"] == m["iters"] and info["restarts"] == m["restarts"]
    assert abs(abs(np.vdot(x, A["lanczos_x"])) - 1.0) <= 1e-10


def test_fuse_roundtrip_is_identity(golden):
    meta, A = golden
    th = _bt(meta, A, "xxz12_b5_theta")
    mat, rec = fuse(th, ((0, 1), (2, 3)))
    assert mat.size == th.size
    # the golden svd input is the fused converged block: same fused legs as any theta here
    ref = meta["xxz12_b5_svdin"]
    assert [list(l.charges) for l in mat.legs] == [l["charges"] for l in ref["legs"]]
    assert [list(l.dims) for l in mat.legs] == [l["dims"] for l in ref["legs"]]


def _xxz(N):
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm, sz, i2 = sp.T.copy(), np.diag([0.5, -0.5]), np.eye(2)
    W = np.zeros((5, 5, 2, 2))
    W[0, 0], W[0, 1], W[0, 2], W[0, 3] = i2, sp, sm, sz
    W[1, 4], W[2, 4], W[3, 4], W[4, 4] = 0.5 * sm, 0.5 * sp, sz, i2
    return [W[0:1] if i == 0 else W[:, 4:5] if i == N - 1 else W for i in range(N)]


def test_block_dmrg_energies_match_reference(golden):
    """XXZ N=12 U(1) chi=16 from the reference's own random start: every sweep's energy."""
    meta, _ = golden
    mpo = O.to_block_mpo(_xxz(12), [[1, -1]] * 12)
    E, M, info = O.dmrg_blocks(mpo, 16, charge=0, n_sweeps=4, seed=1)
    ref = meta["xxz12"]["energies"]
    assert np.allclose(info["energies"], ref, rtol=1e-12, atol=0)


def test_block_mps_start_matches_reference_layout():
    """The random start reproduces the reference's bond sectors (dmrg_small.json, chi=64)."""
    p = os.path.join(GOLDEN, "dmrg_small.json")
    if not os.path.exists(p):
        pytest.skip("dmrg_small.json not generated")
    ref = json.load(open(p))["xxz_n12_chi64"]
    mpo = O.to_block_mpo(_xxz(12), [[1, -1]] * 12)
    E, M, info = O.dmrg_blocks(mpo, 64, charge=0, n_sweeps=4, seed=1)
    assert abs(E - ref["E"]) <= 1e-12 * abs(ref["E"])
    for m, b in zip(M, ref["bonds"]):
        assert list(m.legs[2].charges) == b["charges"] and list(m.legs[2].dims) == b["dims"]


def test_dense_dmrg_tfim_matches_free_fermions(golden):
    meta, _ = golden
    from_ref = meta["tfim10"]
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sz = np.diag([1.0, -1.0])
    W = np.zeros((3, 3, 2, 2))
    W[0, 0], W[0, 1], W[0, 2], W[1, 2], W[2, 2] = np.eye(2), sx, -1.0 * sz, -sx, np.eye(2)
    N = 10
    mpo = [W[0:1] if i == 0 else W[:, 2:3] if i == N - 1 else W for i in range(N)]
    Mb = O.dense_as_blocks(mpo)
    init = O.random_dense_mps(N, 32, 2, np.random.default_rng(0))
    E, M, info = O.dmrg_blocks(Mb, 32, n_sweeps=3, init=init)
    assert abs(E - from_ref["E"]) <= 1e-12 * abs(from_ref["E"])
