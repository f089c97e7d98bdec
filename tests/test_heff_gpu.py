"""GPU parity of the H_eff matvecs and environment updates (through the C ABI) against the
reference's golden vectors and the CPU oracle. FP64: bit-level agreement is not expected
(summation order differs); the bar is 1e-13 relative to the largest entry, as in the reference's
own block-vs-dense tests (tests/test_blocks.py:138-207)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _bt(meta, A, key):
    from tnkit_gb300 import BlockTensor, Leg, layout_of
    m = meta[key]
    lay = layout_of([Leg(tuple(l["charges"]), tuple(l["dims"]), l["sign"]) for l in m["legs"]],
                    m["charge"])
    h = np.ascontiguousarray(A[key], dtype=np.float64)
    return BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_two_site_matches_reference_golden(golden, tag):
    from tnkit_gb300 import ops
    meta, A = golden
    th, L, W1, W2, R = (_bt(meta, A, f"{tag}_{k}") for k in ("theta", "L", "W1", "W2", "R"))
    out = ops.apply_two_site(th, L, W1, W2, R)
    torch.cuda.synchronize()
    assert out.layout is th.layout
    assert _rel(out.data.cpu().numpy(), A[f"{tag}_H2theta"]) <= TOL


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_one_site_and_envs_match_reference_golden(golden, tag):
    from tnkit_gb300 import ops
    meta, A = golden
    L, R1, R, W1, W2, Am, Bm = (_bt(meta, A, f"{tag}_{k}")
                                for k in ("L", "R1", "R", "W1", "W2", "A", "B"))
    assert _rel(ops.apply_one_site(Am, L, W1, R1).data.cpu(), A[f"{tag}_H1A"]) <= TOL
    assert _rel(ops.update_left_env(L, Am, W1).data.cpu(), A[f"{tag}_Lnext"]) <= TOL
    assert _rel(ops.update_right_env(R, Bm, W2).data.cpu(), A[f"{tag}_Rnext"]) <= TOL


def test_dense_matches_reference_golden(golden):
    from tnkit_gb300 import ops, BlockTensor
    from tnkit_gb300.tensor import dense_layout
    _, A = golden

    def bt(x, signs):
        h = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        return BlockTensor(dense_layout(x.shape, signs), torch.as_tensor(h, device="cuda"), h)
    th = bt(A["tfim10_b4_theta"], (1, 1, 1, -1))
    L, R = bt(A["tfim10_b4_L"], (1, -1, -1)), bt(A["tfim10_b4_R"], (-1, 1, 1))
    W1, W2 = bt(A["tfim10_b4_W1"], (1, -1, 1, -1)), bt(A["tfim10_b4_W2"], (1, -1, 1, -1))
    out = ops.apply_two_site(th, L, W1, W2, R)
    assert _rel(out.data.cpu(), A["tfim10_b4_H2theta"].ravel()) <= TOL
    Am, Bm = bt(A["tfim10_b4_A"], (1, 1, -1)), bt(A["tfim10_b4_B"], (1, 1, -1))
    assert _rel(ops.update_left_env(L, Am, W1).data.cpu(), A["tfim10_b4_Lnext"].ravel()) <= TOL
    assert _rel(ops.update_right_env(R, Bm, W2).data.cpu(), A["tfim10_b4_Rnext"].ravel()) <= TOL


def _oracle_two_site(th, L, W1, W2, R):
    from oracle.blocks_np import BT, Leg as OL
    from oracle import dmrg_np as O

    def ob(t):
        legs = [OL(tuple(l.charges), tuple(l.dims), l.sign) for l in t.legs]
        return BT.from_flat(legs, t.charge, t.numpy())
    return O.apply_two_site(ob(th), ob(L), ob(W1), ob(W2), ob(R)).flat()


@pytest.mark.parametrize("scale", [1, 4])
def test_mid_bond_matches_oracle(scale):
    """Sector dims of the chi=1024 mid bond scaled down (uneven, 1..73, not tile multiples)."""
    from tnkit_gb300 import ops, workloads
    dims = [max(1, d // scale) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=scale)
    got = ops.apply_two_site(th, L, W1, W2, R).data.cpu().numpy()
    assert _rel(got, _oracle_two_site(th, L, W1, W2, R)) <= TOL


def test_chi1024_mid_bond_properties():
    """Full size: linearity H(a x + b y) = a Hx + b Hy, and agreement with the oracle."""
    from tnkit_gb300 import ops, workloads
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=3)
    op = ops.TwoSiteOperator(th.layout, L, W1, W2, R)
    x = th.data
    y = torch.randn_like(x)
    a, b = 0.75, -1.25
    lhs = op(a * x + b * y)
    rhs = a * op(x) + b * op(y)
    assert float((lhs - rhs).abs().max() / rhs.abs().max()) <= 1e-13
    got = op(x).cpu().numpy()
    assert _rel(got, _oracle_two_site(th, L, W1, W2, R)) <= TOL


@pytest.mark.parametrize("variant", [0, 1])
def test_two_site_matches_oracle_with_either_fp64_inner_product(variant):
    """The FP64 grouped GEMM's FMA tile (0) and its DMMA tile (mma.sync m8n8k4, 1) give the
    oracle's matvec at a chi=256-like bond and the reference's golden two-site result."""
    from tnkit_gb300 import _lib, ops, workloads
    lib = _lib.lib()
    prev = lib.tnk_gemm_f64_variant(variant)
    try:
        th, L, W1, W2, R = workloads.mid_bond_problem(dims=(3, 24, 61, 80, 61, 24, 3),
                                                      charges=(-6, -4, -2, 0, 2, 4, 6), seed=9)
        got = ops.apply_two_site(th, L, W1, W2, R).data.cpu().numpy()
        ref = _oracle_two_site(th, L, W1, W2, R)
        assert _rel(got, ref) <= TOL
    finally:
        lib.tnk_gemm_f64_variant(prev)
