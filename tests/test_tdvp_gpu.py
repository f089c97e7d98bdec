"""Complex128 path and two-site TDVP on the GPU against the reference's own results
(tests/golden/make_golden.py tdvp): the Krylov exponential on a fixed Hermitian problem, complex
H_eff / environment contractions against the oracle, and the state vector after four TDVP2 steps
of the XXZ N=10 chain from the reference's seeded random block state."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import GOLDEN


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def tg():
    meta = json.load(open(os.path.join(GOLDEN, "tdvp_xxz10.json")))
    A = dict(np.load(os.path.join(GOLDEN, "tdvp_xxz10.npz")))
    return meta, A


@pytest.mark.parametrize("route", ["eigh", "pade"])
def test_lanczos_expm_matches_reference(tg, route):
    """Both routes to exp(tau T) e_1 (the tridiagonal eigendecomposition, and the reference's
    per-iteration scipy expm) give the reference's vector and Krylov dimension."""
    from tnkit_gb300.expm import lanczos_expm
    meta, A = tg
    H = torch.as_tensor(A["expm_H"], device="cuda")
    v = torch.as_tensor(A["expm_v"], device="cuda")
    info = {}
    y = lanczos_expm(lambda x, out: out.copy_(H @ x), v, meta["expm"]["tau_imag"] * 1j,
                     m=meta["expm"]["m"], info=info, route=route)
    ref = A["expm_y"]
    assert info["krylov_dim"] == meta["expm"]["krylov_dim"]
    assert np.abs(y.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("m", [20, 30])
def test_lanczos_expm_fixed_matches_reference(tg, m):
    """The fixed-dimension exponential with every coefficient on the device (no host read
    during the solve, the tridiagonal eigendecomposition by the library's kernel) gives the
    reference's adaptive vector once m is above the dimension the adaptive solver needed."""
    from tnkit_gb300.expm import lanczos_expm_fixed
    meta, A = tg
    H = torch.as_tensor(A["expm_H"], device="cuda")
    v = torch.as_tensor(A["expm_v"], device="cuda")
    assert m > meta["expm"]["krylov_dim"]
    info = {}
    y = lanczos_expm_fixed(lambda x, out: out.copy_(H @ x), v, meta["expm"]["tau_imag"] * 1j,
                           m, info=info)
    ref = A["expm_y"]
    assert info["krylov_dim"] == m
    assert np.abs(y.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


def test_complex_contractions_match_oracle(golden):
    from tnkit_gb300 import BlockTensor, Leg, layout_of, ops
    from oracle.blocks_np import BT, Leg as OL
    from oracle import dmrg_np as O
    meta, A = golden
    tag = "xxz12_b5"
    rng = np.random.default_rng(3)

    def pair(key, real=False):
        m = meta[key]
        lay = layout_of([Leg(tuple(l["charges"]), tuple(l["dims"]), l["sign"]) for l in m["legs"]],
                        m["charge"])
        if real:
            h = np.ascontiguousarray(A[key], dtype=np.float64)
            return BlockTensor(lay, torch.as_tensor(h, device="cuda"), h), BT.from_json(m, h)
        z = rng.standard_normal(lay.size) + 1j * rng.standard_normal(lay.size)
        return BlockTensor(lay, torch.as_tensor(z, device="cuda")), BT.from_json(m, z)
    (th, oth), (L, oL), (R, oR), (R1, oR1) = (pair(f"{tag}_{k}") for k in ("theta", "L", "R", "R1"))
    (W1, oW1), (W2, oW2) = pair(f"{tag}_W1", True), pair(f"{tag}_W2", True)
    (Am, oA), (Bm, oB) = pair(f"{tag}_A"), pair(f"{tag}_B")
    rel = lambda a, b: float(np.abs(a - b).max() / np.abs(b).max())
    assert rel(ops.apply_two_site(th, L, W1, W2, R).data.cpu().numpy(),
               O.apply_two_site(oth, oL, oW1, oW2, oR).flat()) <= 1e-13
    assert rel(ops.apply_one_site(Am, L, W1, R1).data.cpu().numpy(),
               O.apply_one_site(oA, oL, oW1, oR1).flat()) <= 1e-13
    assert rel(ops.update_left_env(L, Am, W1).data.cpu().numpy(),
               O.update_left_env(oL, oA, oW1).flat()) <= 1e-13
    assert rel(ops.update_right_env(R, Bm, W2).data.cpu().numpy(),
               O.update_right_env(oR, oB, oW2).flat()) <= 1e-13


@pytest.mark.parametrize("fast_expm", [None, 20, "auto"])
def test_tdvp2_state_matches_reference(tg, fast_expm):
    """Four TDVP2 steps from the reference's seeded state: its final state vector and bonds,
    with the adaptive Krylov exponential and with the fixed-dimension one (a fixed m, and m
    calibrated on the first step: the reference's fast_expm)."""
    from tnkit_gb300 import BlockTensor, Leg, layout_of, workloads
    from tnkit_gb300.mpo import to_block_mpo
    from tnkit_gb300.tdvp import tdvp2_evolve, dense_vector
    meta, A = tg
    p = meta["params"]
    N = p["N"]
    mps = []
    for i in range(N):
        m = meta[f"init_{i}"]
        lay = layout_of([Leg(tuple(l["charges"]), tuple(l["dims"]), l["sign"]) for l in m["legs"]],
                        m["charge"])
        mps.append(BlockTensor(lay, torch.as_tensor(A[f"init_{i}"], device="cuda")))
    v0 = dense_vector(mps)
    assert np.abs(v0 - A["init_vector"]).max() <= 1e-13 * np.abs(A["init_vector"]).max()
    Wb = to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N)[0]
    prof = {}
    out, rec = tdvp2_evolve(mps, Wb, p["chi"], p["dt"], p["n_steps"], profile=prof,
                            fast_expm=fast_expm)
    v = dense_vector(out)
    ref = A["final_vector"]
    assert abs(abs(np.vdot(ref, v)) / (np.linalg.norm(ref) * np.linalg.norm(v)) - 1) <= 1e-11
    assert np.abs(v - ref).max() <= 1e-10 * np.abs(ref).max()
    for m, b in zip(out, meta["final_bonds"]):
        assert list(m.legs[2].charges) == b["charges"] and list(m.legs[2].dims) == b["dims"]
