"""The tensor-core (tcgen05, TF32) two-site matvec and the mixed-precision local solve.

Tolerances: the split-TF32 matvec (three MMAs of TF32 hi/lo parts, FP32 accumulation) agrees with
the FP64 matvec to 1e-4 relative to the largest entry (typically ~1e-6); plain TF32 to 3e-2.
The mixed local solve (tensor-core Lanczos, then FP64 polish to the same residual tolerance) must
reach the FP64 solve's eigenvalue to |dE| <= 1e-10."""
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


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("scale", [8, 2, 1])
@pytest.mark.parametrize("passes,tol", [(3, 1e-4), (1, 3e-2)])
def test_tc_matvec_matches_fp64(scale, passes, tol):
    from tnkit_gb300 import ops, workloads
    from tnkit_gb300.mixed import TwoSiteOperatorTC
    dims = [max(1, d // scale) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=20 + scale)
    op64 = ops.TwoSiteOperator(th.layout, L, W1, W2, R)
    optc = TwoSiteOperatorTC(th.layout, L, W1, W2, R, passes=passes)
    ref = op64(th.data)
    for _ in range(2):                  # twice: staging buffers are reused between calls
        got = optc(th.data)
    torch.cuda.synchronize()
    optc.check_device_error()
    assert torch.isfinite(got).all()
    assert _rel(got, ref) <= tol, _rel(got, ref)


@pytest.mark.parametrize("passes", [3, 1])
def test_tc_persistent_schedule_equals_one_tile_per_cta(passes):
    """Stages with more tiles than SMs run persistent CTAs with two TMEM accumulators when
    tnk_tc_schedule(1) is set: the same MMAs per tile in the same order, so the result is the
    one-tile-per-CTA result bit for bit -- on the chi=1024 mid bond (294 stage-1 tiles) and on
    a 48-chain batched plan."""
    from tnkit_gb300 import _lib, batch as B, ops, workloads
    from tnkit_gb300.mixed import TwoSiteOperatorTC
    lib = _lib.lib()
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=31)
    optc = TwoSiteOperatorTC(th.layout, L, W1, W2, R, passes=passes)
    opb = B.BatchedTwoSiteOperator(B.batch_problems(48, seed=2), precision="tc")
    xb = torch.randn(opb.n, dtype=torch.float64, device="cuda")
    assert len(optc.host.tiles1) > 152
    prev = lib.tnk_tc_schedule(0)
    try:
        a = optc(th.data)
        ab = opb(xb)
        lib.tnk_tc_schedule(1)
        for _ in range(2):
            b = optc(th.data)
            bb = opb(xb)
        torch.cuda.synchronize()
    finally:
        lib.tnk_tc_schedule(prev)
    optc.check_device_error()
    opb.tc.check_device_error()
    assert torch.equal(a, b) and torch.equal(ab, bb)
    if passes == 3:
        ref = ops.TwoSiteOperator(th.layout, L, W1, W2, R)(th.data)
        assert _rel(b, ref) <= 1e-4


def test_tc_shared_memory_split_matches_staged_split():
    """passes=4 (operands staged once as FP32, the TF32 hi/lo parts formed in shared memory by
    the GEMM) is as accurate as the staged split (passes=3) against the FP64 matvec -- the
    chi=1024 mid bond (128 x 128 and 128 x 64 tiles) and a 48-chain batched plan. The two differ
    in the lo parts of FP64-sourced operands (the staged split rounds the FP64 residual x - hi,
    the shared-memory split the FP32 one), at ~1e-7 of the result."""
    from tnkit_gb300 import batch as B, ops, workloads
    from tnkit_gb300.mixed import TwoSiteOperatorTC
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=41)
    ref = ops.TwoSiteOperator(th.layout, L, W1, W2, R)(th.data)
    a = TwoSiteOperatorTC(th.layout, L, W1, W2, R, passes=3)(th.data)
    op4 = TwoSiteOperatorTC(th.layout, L, W1, W2, R, passes=4)
    b = op4(th.data)
    probs = B.batch_problems(48, seed=2)
    p3 = B.BatchedTwoSiteOperator(probs, precision="tc")
    xb = torch.randn(p3.n, dtype=torch.float64, device="cuda")
    ab = p3(xb)
    p4 = B.BatchedTwoSiteOperator(probs, precision="tc", tc_passes=4)
    bb = p4(xb)
    bref = B.BatchedTwoSiteOperator(probs, precision="f64")(xb)
    torch.cuda.synchronize()
    op4.check_device_error()
    p4.tc.check_device_error()
    assert _rel(b, ref) <= 1e-4 and _rel(bb, bref) <= 1e-4
    assert _rel(b, ref) <= 2 * _rel(a, ref) + 1e-7
    assert _rel(b, a) <= 1e-5 and _rel(bb, ab) <= 1e-5


def test_tc_matvec_golden_problem(golden):
    """The reference's own (converged-state) XXZ N=12 local problem."""
    from tnkit_gb300 import BlockTensor, Leg, layout_of
    from tnkit_gb300.mixed import TwoSiteOperatorTC
    meta, A = golden

    def bt(key):
        m = meta[key]
        lay = layout_of([Leg(tuple(l["charges"]), tuple(l["dims"]), l["sign"]) for l in m["legs"]],
                        m["charge"])
        h = np.ascontiguousarray(A[key], dtype=np.float64)
        return BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    tag = "xxz12_b5"
    th, L, W1, W2, R = (bt(f"{tag}_{k}") for k in ("theta", "L", "W1", "W2", "R"))
    got = TwoSiteOperatorTC(th.layout, L, W1, W2, R)(th.data)
    ref = torch.as_tensor(A[f"{tag}_H2theta"], device="cuda")
    assert _rel(got, ref) <= 1e-4


def _xxz_blocks(N):
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import to_block_mpo
    return to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N)[0]


@pytest.mark.parametrize("N,chi,sweeps", [(12, 16, 4), (32, 64, 3)])
def test_mixed_dmrg_matches_fp64_dmrg(N, chi, sweeps):
    """Whole sweeps with tensor-core Lanczos + FP64 polish against the plain FP64 sweep from
    the same start: |dE| <= 1e-10 at every sweep, and most matvecs on the tensor cores."""
    from tnkit_gb300.dmrg import dmrg
    kw = dict(charge=0, seed=1, n_sweeps=sweeps, tol=0, rtol=0, expand=0)
    E64, _, i64 = dmrg(_xxz_blocks(N), chi, **kw)
    Em, _, im = dmrg(_xxz_blocks(N), chi, precision="mixed", **kw)
    assert abs(Em - E64) <= 1e-10, (Em, E64)
    assert np.allclose(im["energies"], i64["energies"], rtol=0, atol=1e-10)
    assert im["mixed_counts"]["lo"] > 0


@pytest.mark.parametrize("scale", [4, 1])
def test_float_float_matvec_matches_fp64(scale):
    """The float-float grouped GEMM (double-FP32 on the FP32 cores) on the same plan: within
    1e-12 of the FP64 matvec, relative to the largest entry."""
    from tnkit_gb300 import ops, workloads
    dims = [max(1, d // scale) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=40 + scale)
    ref = ops.TwoSiteOperator(th.layout, L, W1, W2, R)(th.data)
    got = ops.TwoSiteOperator(th.layout, L, W1, W2, R, precision="ff")(th.data)
    assert _rel(got, ref) <= 1e-12, _rel(got, ref)


@pytest.mark.parametrize("prec", ["ff", "mixed-ff"])
def test_ff_dmrg_matches_reference(prec):
    """Whole sweeps on the float-float matvec (alone, or as the polish after tensor-core
    Lanczos): the reference's energies to 1e-12 relative."""
    import json, os
    from conftest import GOLDEN
    from tnkit_gb300.dmrg import dmrg
    ref = json.load(open(os.path.join(GOLDEN, "dmrg_small.json")))["xxz_n64_chi64"]
    E, M, info = dmrg(_xxz_blocks(64), 64, charge=0, seed=1, n_sweeps=len(ref["energies"]),
                      tol=0, rtol=0, expand=0, precision=prec)
    assert abs(E - ref["E"]) <= 1e-12 * abs(ref["E"]), (E, ref["E"])


@pytest.mark.parametrize("scale", [4, 1])
def test_float_float_env_updates_match_fp64(scale):
    """Left and right environment updates in float-float against FP64 at the chi=1024 mid-bond
    sectors (scaled down by `scale`): ~1e-14 relative to the largest entry."""
    from tnkit_gb300 import ops, workloads
    from tnkit_gb300.layout import Leg, layout_of
    from tnkit_gb300.tensor import BlockTensor
    dims = [max(1, d // scale) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=11)
    bl, phys = th.layout.legs[0], th.layout.legs[1]
    # the neighbouring bond: odd charges -9..9 (one spin more or less), dims between the mid's
    odd = tuple(range(-9, 10, 2))
    dodd = (dims[0],) + tuple(max(1, (a + b) // 2) for a, b in zip(dims, dims[1:])) + (dims[-1],)
    rng = np.random.default_rng(3)
    A_l = layout_of((bl, phys, Leg(odd, dodd, -1)), 0)
    A = BlockTensor(A_l, torch.as_tensor(rng.standard_normal(A_l.size), device="cuda"))
    B_l = layout_of((Leg(odd, dodd, 1), phys, bl.flip()), 0)
    B = BlockTensor(B_l, torch.as_tensor(rng.standard_normal(B_l.size), device="cuda"))
    for f, env, site, W in ((ops.update_left_env, L, A, W1), (ops.update_right_env, R, B, W2)):
        ref = f(env, site, W).data
        got = f(env, site, W, precision="ff").data
        assert got.shape == ref.shape
        assert _rel(got, ref) <= 1e-13, (f.__name__, _rel(got, ref))


@pytest.mark.parametrize("prec,polish,mode", [("mixed-ff", 2, "lanczos"),
                                              ("mixed-ff", 1, "lanczos"),
                                              ("mixed", 1, "lanczos"), ("mixed", 1, "refine"),
                                              ("mixed-ff", 1, "refine")])
def test_sweep_schedule_reaches_fp64_energy(prec, polish, mode):
    """mixed_schedule='sweep': the opening sweeps on the tensor cores alone, the last one or two
    polished (float-float or FP64; by Lanczos, or by defect correction with tensor-core
    correction solves), end within 1e-10 of the FP64 run's energy."""
    from tnkit_gb300.dmrg import dmrg
    kw = dict(charge=0, seed=1, n_sweeps=6, tol=0, rtol=0, expand=0)
    E64, _, _ = dmrg(_xxz_blocks(32), 64, **kw)
    E, M, info = dmrg(_xxz_blocks(32), 64, precision=prec, mixed_schedule="sweep",
                      polish_sweeps=polish, polish_mode=mode, **kw)
    assert info["mixed_counts"]["lo"] > info["mixed_counts"]["hi"] > 0
    assert abs(E - E64) <= 1e-10, (E, E64)              # absolute, as the target states


def test_refine_ground_reaches_fp64_eigenpair():
    """Defect correction with the tensor-core operator as the inner solver reaches the FP64
    ground state of a small U(1) local problem made symmetric, (H + H^T) / 2, in a few outer
    steps, from a start 1e-3 away."""
    from tnkit_gb300 import ops, workloads
    from tnkit_gb300.mixed import TwoSiteOperatorTC, refine_ground
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=(2, 6, 10, 6, 2),
                                                  charges=(-4, -2, 0, 2, 4), seed=4)
    n = th.layout.size
    op = ops.TwoSiteOperator(th.layout, L, W1, W2, R)
    tc = TwoSiteOperatorTC(th.layout, L, W1, W2, R)
    # a dense symmetric stand-in built from the operator, for the reference eigenpair
    E = torch.eye(n, dtype=torch.float64, device="cuda")
    H = torch.stack([op(E[:, j].contiguous()) for j in range(n)], 1) if n <= 4000 else None
    if H is None:
        pytest.skip("problem too large for the dense check")
    Hs = 0.5 * (H + H.T)
    ev, evec = torch.linalg.eigh(Hs)
    sym64 = lambda x, out: out.copy_(Hs @ x)
    sym_lo = lambda x, out: out.copy_(0.5 * (tc(x) + (H.T @ x)))      # ~1e-6 away from Hs
    x0 = evec[:, 0] + 1e-3 * torch.randn(n, dtype=torch.float64, device="cuda")
    th_, x, info = refine_ground(sym64, sym_lo, x0, tol=1e-10)
    tc.check_device_error()
    assert info["residual"] < 1e-10 and info["outer"] <= 3, info
    assert abs(th_ - float(ev[0])) <= 1e-12 * abs(float(ev[0]))
    assert abs(abs(float(torch.dot(x, evec[:, 0]))) - 1.0) <= 1e-10
