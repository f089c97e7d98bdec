"""The GPU Lanczos and the whole two-site DMRG sweep against the reference's own results
(golden energies from tests/golden/make_golden.py) and exact answers."""
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


def test_lanczos_restart_matches_reference(golden):
    """The reference's thick-restart Lanczos known answer: same eigenvalue, iteration and
    restart counts (tnkit/eigensolver.py:507-674 on a 300 x 300 symmetric matrix)."""
    from tnkit_gb300.lanczos import lanczos_ground_restart
    meta, A = golden
    m = meta["lanczos"]
    H = torch.as_tensor(A["lanczos_H"], device="cuda")
    v0 = torch.as_tensor(A["lanczos_v0"], device="cuda")
    e, x, info = lanczos_ground_restart(lambda v, out: out.copy_(H @ v), v0, tol=m["tol"],
                                        max_iter=m["max_iter"], m=m["m"], k=m["k"])
    assert abs(e - m["e"]) <= 1e-12 * abs(m["e"])
    assert info["iters"] == m["iters"] and info["restarts"] == m["restarts"]
    xr = A["lanczos_x"]
    assert abs(abs(float(np.dot(x.cpu().numpy(), xr))) - 1.0) <= 1e-10


def _xxz_blocks(N):
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import to_block_mpo
    return to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N)[0]


def test_block_dmrg_xxz12_every_sweep_matches_reference(golden):
    """Same random start as the reference (seed 1), same sweep: every sweep's energy."""
    from tnkit_gb300.dmrg import dmrg
    meta, _ = golden
    E, M, info = dmrg(_xxz_blocks(12), 16, charge=0, seed=1, n_sweeps=4, tol=0, rtol=0, expand=0)
    ref = meta["xxz12"]["energies"]
    assert np.allclose(info["energies"], ref, rtol=1e-12, atol=0), (info["energies"], ref)
    assert [m.legs[2].charges for m in M][-1] == (0,)


@pytest.mark.parametrize("N,chi", [(12, 64), (64, 64)])
def test_block_dmrg_matches_reference_runs(N, chi):
    from tnkit_gb300.dmrg import dmrg
    ref = json.load(open(os.path.join(GOLDEN, "dmrg_small.json")))[f"xxz_n{N}_chi{chi}"]
    sweeps = len(ref["energies"])
    E, M, info = dmrg(_xxz_blocks(N), chi, charge=0, seed=1, n_sweeps=sweeps, tol=0, rtol=0,
                      expand=0)
    assert abs(E - ref["E"]) <= 1e-12 * abs(ref["E"]), (E, ref["E"])
    for m, b in zip(M, ref["bonds"]):
        assert list(m.legs[2].dims) == b["dims"] and list(m.legs[2].charges) == b["charges"]


def test_dense_dmrg_tfim_free_fermion():
    from tnkit_gb300 import workloads
    from tnkit_gb300.dmrg import dmrg
    ref = json.load(open(os.path.join(GOLDEN, "dmrg_small.json")))["c1_tfim_n10_chi32"]
    E, M, info = dmrg(workloads.tfim_mpo(10, 1.0), 32, n_sweeps=10, tol=0, rtol=0, seed=0)
    assert abs(E - ref["free_fermion"]) <= 1e-12 * abs(ref["free_fermion"])
    assert abs(E - ref["E"]) <= 1e-12 * abs(ref["E"])
    assert not info["blocks"]


@pytest.mark.parametrize("N,chi", [(12, 64), (64, 64)])
def test_block_dmrg_gram_truncation_matches_reference(N, chi):
    """The Gram-matrix truncation (eigh + QR per sector, concurrent over sectors) reaches the
    reference's exact-SVD energies to 1e-10."""
    from tnkit_gb300.dmrg import dmrg
    ref = json.load(open(os.path.join(GOLDEN, "dmrg_small.json")))[f"xxz_n{N}_chi{chi}"]
    E, M, info = dmrg(_xxz_blocks(N), chi, charge=0, seed=1, n_sweeps=len(ref["energies"]),
                      tol=0, rtol=0, expand=0, svd_method="gram")
    assert abs(E - ref["E"]) <= 1e-10, (E, ref["E"])


@pytest.mark.parametrize("N,chi", [(6, 16), (8, 32)])
def test_hubbard_u1xu1_every_sweep_matches_reference(N, chi):
    """The Fermi-Hubbard chain under U(1) x U(1) (N_up, N_dn) blocks, half filling: the same
    seeded start as the reference, its final energy to 1e-12 relative and every sweep's to
    1e-10 (a sweep still far from convergence depends on where each local Lanczos stops, at a
    1e-9 residual), every bond's (N_up, N_dn) sectors at the end."""
    from tnkit_gb300 import workloads
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.mpo import to_block_mpo
    ref = json.load(open(os.path.join(GOLDEN, "hubbard_u1u1.json")))["runs"][f"n{N}_chi{chi}"]
    Wb, _ = to_block_mpo(workloads.hubbard_mpo(N), [workloads.HUBBARD_SITE_CHARGES] * N)
    E, M, info = dmrg(Wb, chi, charge=(N // 2, N // 2), seed=1, n_sweeps=len(ref["energies"]),
                      tol=0, rtol=0, expand=0)
    assert abs(E - ref["E"]) <= 1e-12 * abs(ref["E"]), (E, ref["E"])
    assert np.allclose(info["energies"], ref["energies"], rtol=1e-10, atol=0), \
        (info["energies"], ref["energies"])
    for m, b in zip(M, ref["bonds"]):
        assert [list(c) for c in m.legs[2].charges] == b["charges"]
        assert list(m.legs[2].dims) == b["dims"]
