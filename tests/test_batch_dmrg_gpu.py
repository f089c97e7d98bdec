"""Lockstep DMRG of many chains (tnkit_gb300.batch_dmrg): the batched Lanczos against dense
eigensolvers on independent matrices of different sizes, and a batch of dense Ising and U(1)
XXZ chains of different lengths and bond dimensions against the same chains run one by one
with `dmrg` (the oracle: a loop of independent calls) and against the reference's golden
free-fermion energy."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


@pytest.mark.parametrize("segmented", [True, False])
def test_batched_lanczos_matches_eigvalsh(segmented):
    """Every chain's lowest eigenpair, with the Gram-Schmidt passes and normalisations as one
    segmented launch for all chains (tnk_cgs_pass_seg_f64) or one launch per chain."""
    from tnkit_gb300.batch_dmrg import lanczos_ground_batched
    rng = np.random.default_rng(5)
    sizes = [1, 3, 7, 40, 120, 300, 55]
    Hs = []
    for n in sizes:
        A = rng.standard_normal((n, n))
        Hs.append((A + A.T) / 2)
    off = np.concatenate([[0], np.cumsum(sizes)])
    Hd = [torch.as_tensor(H, device="cuda") for H in Hs]

    def op(x, out):
        for H, a, b in zip(Hd, off[:-1], off[1:]):
            torch.mv(H, x[a:b], out=out[a:b])
        return out
    x0 = torch.as_tensor(rng.standard_normal(off[-1]), device="cuda")
    E, X, info = lanczos_ground_batched(op, x0, off, tol=1e-10, max_iter=600, m=30, k=8,
                                        segmented=segmented)
    assert info["converged"].all() and info["restarts"] > 0
    for H, e, a, b in zip(Hs, E, off[:-1], off[1:]):
        ev, evec = np.linalg.eigh(H)
        assert abs(e - ev[0]) <= 1e-9 * max(1.0, abs(ev[0]))
        x = X[a:b].cpu().numpy()
        assert abs(np.linalg.norm(x) - 1.0) <= 1e-12
        assert abs(abs(x @ evec[:, 0]) - 1.0) <= 1e-8


@pytest.mark.parametrize("precision,pipeline", [("f64", True), ("ff", True), ("f64", False),
                                                ("mixed", False)])
def test_dmrg_batch_matches_independent_runs(precision, pipeline):
    from tnkit_gb300 import workloads
    from tnkit_gb300.batch_dmrg import dmrg_batch
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.mpo import to_block_mpo
    xxz = lambda N, d: to_block_mpo(workloads.xxz_mpo(N, d), [[1, -1]] * N)[0]
    specs = [("tfim", 10, 32, 1.0, 0), ("xxz", 12, 16, 1.0, 1), ("tfim", 8, 8, 0.7, 3),
             ("xxz", 16, 32, 0.5, 2)]
    mk = lambda m, N, g: workloads.tfim_mpo(N, g) if m == "tfim" else xxz(N, g)
    sweeps = 6
    Eb, Mb, info = dmrg_batch([mk(m, N, g) for m, N, _, g, _ in specs],
                              [chi for _, _, chi, _, _ in specs],
                              charges=[None if m == "tfim" else 0 for m, *_ in specs],
                              seeds=[s for *_, s in specs], n_sweeps=sweeps, tol=0, rtol=0,
                              expand=0, precision=precision, pipeline=pipeline)
    assert info["rounds"] == sweeps * 2 * (16 - 1)
    for (m, N, chi, g, seed), e, es in zip(specs, Eb, info["energies"]):
        assert len(es) == sweeps
        kw = dict(seed=seed, n_sweeps=sweeps, tol=0, rtol=0, expand=0)
        if m == "xxz":
            kw["charge"] = 0
        E1, _, _ = dmrg(mk(m, N, g), chi, **kw)
        assert abs(e - E1) <= 1e-10 * abs(E1), (m, N, e, E1)
    ref = json.load(open(os.path.join(GOLDEN, "dmrg_small.json")))["c1_tfim_n10_chi32"]
    assert abs(Eb[0] - ref["free_fermion"]) <= 1e-11 * abs(ref["free_fermion"])


def test_segmented_passes_equal_per_chain_passes():
    """One segmented launch per Gram-Schmidt pass gives each chain the per-chain pass's
    coefficients and vector (only the order of partial sums differs: 1e-14)."""
    from tnkit_gb300.batch_dmrg import _Segments, _MAXNV
    rng = np.random.default_rng(8)
    sizes = [5, 1000, 129, 40000, 7, 3000]
    off = np.concatenate([[0], np.cumsum(sizes)])
    n = int(off[-1])
    nv = 9
    V = torch.as_tensor(rng.standard_normal((nv, n)), device="cuda")
    w0 = torch.as_tensor(rng.standard_normal(n), device="cuda")
    act = [0, 1, 3, 5]
    A = _Segments(off, n, torch.device("cuda"), segmented=True)
    B = _Segments(off, n, torch.device("cuda"), segmented=False)
    wa, wb = w0.clone(), w0.clone()
    A.cgs2_all(V, nv, wa, act)
    for c in act:
        B.cgs2(V, nv, wb, c)
    ra, rb = A.read().copy(), B.read().copy()
    for c in act:
        a, b = off[c], off[c + 1]
        assert np.allclose(ra[c, :1 + 2 * _MAXNV], rb[c, :1 + 2 * _MAXNV], rtol=1e-13,
                           atol=1e-13 * np.abs(rb[c]).max())
        assert torch.allclose(wa[a:b], wb[a:b], rtol=0, atol=1e-13 * float(wb[a:b].abs().max()))
    for c in (2, 4):                     # chains not listed are untouched
        a, b = off[c], off[c + 1]
        assert torch.equal(wa[a:b], w0[a:b])
    ya, yb = torch.zeros_like(w0), torch.zeros_like(w0)
    A.scale_div_all(wa, ya, act)
    for c in act:
        B.scale_div(wb, yb, c)
    assert torch.allclose(ya, yb, rtol=0, atol=1e-12 * float(yb.abs().max()))
