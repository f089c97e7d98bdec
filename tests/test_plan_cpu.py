"""Host planners (tnkit_gb300.plan) checked on the CPU: their task tables, run through a numpy
interpreter of the kernel semantics, reproduce the reference's golden outputs and the oracle."""
import numpy as np
import pytest

from tnkit_gb300 import plan as P
from tnkit_gb300.layout import Leg, canonical, layout_of
from oracle.blocks_np import BT
from oracle import dmrg_np as O
from table_interp import run_plan3, run_gemm, run_comb


def lay(meta):
    return layout_of([Leg(tuple(l["charges"]), tuple(l["dims"]), l["sign"]) for l in meta["legs"]],
                     meta["charge"])


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_two_site_plan_matches_reference(golden, tag):
    meta, A = golden
    g = lambda k: (lay(meta[f"{tag}_{k}"]), A[f"{tag}_{k}"])
    (Ll, Ld), (Rl, Rd), (W1l, W1d), (W2l, W2d), (Tl, Td) = (g(k) for k in ("L", "R", "W1", "W2", "theta"))
    p = P.plan_apply(Tl, Ll, [(W1l, W1d), (W2l, W2d)], Rl)
    assert p.out_layout.size == Tl.size and p.out_layout is Tl
    out = run_plan3(p, Ld, Td, Rd)
    assert _rel(out, A[f"{tag}_H2theta"]) <= 1e-13
    ref_macs = P.two_site_ref_macs(Tl, Ll, W1l, W2l, Rl)
    th = BT.from_json(meta[f"{tag}_theta"], Td)
    L = BT.from_json(meta[f"{tag}_L"], Ld)
    W1, W2 = BT.from_json(meta[f"{tag}_W1"], W1d), BT.from_json(meta[f"{tag}_W2"], W2d)
    R = BT.from_json(meta[f"{tag}_R"], Rd)
    assert ref_macs == O.two_site_macs(th, L, W1, W2, R)
    assert p.macs <= ref_macs


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_one_site_and_env_plans_match_reference(golden, tag):
    meta, A = golden
    g = lambda k: (lay(meta[f"{tag}_{k}"]), A[f"{tag}_{k}"])
    (Ll, Ld), (R1l, R1d), (Rl, Rd) = g("L"), g("R1"), g("R")
    (W1l, W1d), (W2l, W2d), (Al, Ad), (Bl, Bd) = g("W1"), g("W2"), g("A"), g("B")
    p1 = P.plan_apply(Al, Ll, [(W1l, W1d)], R1l)
    assert _rel(run_plan3(p1, Ld, Ad, R1d), A[f"{tag}_H1A"]) <= 1e-13
    pl = P.plan_left_env(Ll, Al, (W1l, W1d))
    got = run_plan3(pl, Ad, Ld, Ad)
    ref = BT.from_json(meta[f"{tag}_A"], Ad)
    want = O.update_left_env(BT.from_json(meta[f"{tag}_L"], Ld), ref,
                             BT.from_json(meta[f"{tag}_W1"], W1d))
    assert [l.charges for l in pl.out_layout.legs] == [l.charges for l in want.legs]
    assert _rel(got, A[f"{tag}_Lnext"]) <= 1e-13
    pr = P.plan_right_env(Rl, Bl, (W2l, W2d))
    assert _rel(run_plan3(pr, Bd, Rd, Bd), A[f"{tag}_Rnext"]) <= 1e-13


def _dense_layout(shape, signs):
    return canonical(tuple(Leg((0,), (n,), s) for n, s in zip(shape, signs)), 0)


def test_dense_plans_match_reference(golden):
    _, A = golden
    th, L, W1, W2, R = (A[f"tfim10_b4_{k}"] for k in ("theta", "L", "W1", "W2", "R"))
    Tl = _dense_layout(th.shape, (1, 1, 1, -1))
    Ll = _dense_layout(L.shape, (1, -1, -1))
    Rl = _dense_layout(R.shape, (-1, 1, 1))
    W1l = _dense_layout(W1.shape, (1, -1, 1, -1))
    W2l = _dense_layout(W2.shape, (1, -1, 1, -1))
    p = P.plan_apply(Tl, Ll, [(W1l, W1.ravel()), (W2l, W2.ravel())], Rl)
    out = run_plan3(p, L.ravel(), th.ravel(), R.ravel())
    assert _rel(out, A["tfim10_b4_H2theta"].ravel()) <= 1e-13
    Am, Bm = A["tfim10_b4_A"], A["tfim10_b4_B"]
    Al = _dense_layout(Am.shape, (1, 1, -1))
    Bl = _dense_layout(Bm.shape, (1, 1, -1))
    pl = P.plan_left_env(Ll, Al, (W1l, W1.ravel()))
    assert _rel(run_plan3(pl, Am.ravel(), L.ravel(), Am.ravel()),
                A["tfim10_b4_Lnext"].ravel()) <= 1e-13
    pr = P.plan_right_env(Rl, Bl, (W2l, W2.ravel()))
    assert _rel(run_plan3(pr, Bm.ravel(), R.ravel(), Bm.ravel()),
                A["tfim10_b4_Rnext"].ravel()) <= 1e-13


def test_tensordot_fuse_split_plans(golden):
    meta, A = golden
    Al, Bl = lay(meta["xxz12_b5_A"]), lay(meta["xxz12_b5_B"])
    # a theta from two site tensors with a matching bond: use A and a random right tensor
    a = BT.from_json(meta["xxz12_b5_A"], A["xxz12_b5_A"])
    rng = np.random.default_rng(0)
    bl = canonical((Al.legs[2].flip(), Al.legs[1], Leg((-1, 1), (2, 3), -1)), 0)
    bd = rng.standard_normal(bl.size)
    pt = P.plan_tensordot(Al, bl, 1)
    out = np.zeros(pt.out_layout.size)
    run_gemm(pt.g, [A["xxz12_b5_A"], bd, None, None], out)
    bo = BT.from_flat([Leg(l.charges, l.dims, l.sign) for l in bl.legs], 0, bd)
    from oracle.blocks_np import Leg as OLeg, tensordot as otd, fuse as ofuse
    bo = BT.from_flat([OLeg(tuple(l.charges), tuple(l.dims), l.sign) for l in bl.legs], 0, bd)
    ref = otd(a, bo, (2,), (0,))
    assert _rel(out, ref.flat()) <= 1e-13
    # fuse the 4-leg result into a matrix and split rows/cols back
    info = P.FuseInfo(pt.out_layout, 2)
    pf = P.plan_fuse(info)
    mat = np.zeros(info.matrix.size)
    run_comb(pf.c, out, mat)
    mref, _ = ofuse(ref, ((0, 1), (2, 3)))
    assert np.array_equal(mat, mref.flat())
    assert [l.dims for l in info.matrix.legs] == [l.dims for l in mref.legs]


@pytest.mark.parametrize("passes,tol", [(3, 2e-5), (1, 3e-2)])
def test_tensor_core_plan_relayout(passes, tol):
    """The tensor-core re-layout (staged K-major blocks, transposed theta, padded Z) reproduces
    the FP64 matvec to the accuracy of split / plain TF32, on uneven scaled mid-bond sectors."""
    from tnkit_gb300 import workloads
    from table_interp import run_tc_plan
    dims = [max(1, d // 8) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=5, device="cpu")
    hp = P.plan_apply(th.layout, L.layout, [(W1.layout, W1.host), (W2.layout, W2.host)], R.layout)
    ref = run_plan3(hp, L.host, th.host, R.host)
    tc = P.HostPlanTC(hp, th.layout, L.layout, R.layout)
    got = run_tc_plan(tc, L.host, th.host, R.host, passes=passes)
    assert _rel(got, ref) <= tol
    for off, r, c, ld in tc.maps:
        assert off % P.TC_ALIGN == 0 and (ld * 4) % 16 == 0 and ld >= c
    assert tc.stage_elems % P.TC_ALIGN == 0


def _cplx(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def test_complex_plans_match_oracle(golden):
    """Complex128 operands through the interleaved re/im expansion of the real plans, against
    the oracle's complex contractions (the conjugated site tensor of the environment updates
    included)."""
    from oracle.blocks_np import BT, Leg as OL
    meta, A = golden
    tag = "xxz12_b5"
    g = lambda k: lay(meta[f"{tag}_{k}"])
    Ll, Rl, W1l, W2l, Tl, Al, Bl, R1l = (g(k) for k in ("L", "R", "W1", "W2", "theta", "A", "B",
                                                          "R1"))
    W1d, W2d = A[f"{tag}_W1"], A[f"{tag}_W2"]
    rng = np.random.default_rng(9)
    L, R, th, Am, Bm, R1 = (_cplx(rng, x.size) for x in (Ll, Rl, Tl, Al, Bl, R1l))
    iv = lambda z: np.stack([z.real, z.imag], -1).reshape(-1)      # interleaved view
    cv = lambda d: d[0::2] + 1j * d[1::2]
    ob = lambda l, d: BT.from_flat([OL(tuple(x.charges), tuple(x.dims), x.sign) for x in l.legs],
                                   l.charge, d)
    W1, W2 = ob(W1l, W1d), ob(W2l, W2d)
    hp = P.plan_apply(Tl, Ll, [(W1l, W1d), (W2l, W2d)], Rl)
    got = cv(run_plan3(P.ComplexPlan3(hp), iv(L), iv(th), iv(R)))
    ref = O.apply_two_site(ob(Tl, th), ob(Ll, L), W1, W2, ob(Rl, R)).flat()
    assert _rel(got, ref) <= 1e-13
    p1 = P.plan_apply(Al, Ll, [(W1l, W1d)], R1l)
    got = cv(run_plan3(P.ComplexPlan3(p1), iv(L), iv(Am), iv(R1)))
    assert _rel(got, O.apply_one_site(ob(Al, Am), ob(Ll, L), W1, ob(R1l, R1)).flat()) <= 1e-13
    pl = P.plan_left_env(Ll, Al, (W1l, W1d))
    got = cv(run_plan3(P.ComplexPlan3(pl), iv(Am), iv(L), iv(Am)))
    assert _rel(got, O.update_left_env(ob(Ll, L), ob(Al, Am), W1).flat()) <= 1e-13
    pr = P.plan_right_env(Rl, Bl, (W2l, W2d))
    got = cv(run_plan3(P.ComplexPlan3(pr), iv(Bm), iv(R), iv(Bm)))
    assert _rel(got, O.update_right_env(ob(Rl, R), ob(Bl, Bm), W2).flat()) <= 1e-13


def test_split_k_stage_balances_and_matches():
    """The split of long stage-3 tiles along K (partials in the workspace, stage 4 sums them):
    the same result, and no tile longer than a few times the average work per resident CTA."""
    from tnkit_gb300 import workloads
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=6, device="cpu")
    hp = P.plan_apply(th.layout, L.layout, [(W1.layout, W1.host), (W2.layout, W2.host)], R.layout)
    assert len(hp.c4[0]) > 0 and hp.ws2 > hp.ws2_unsplit
    import copy
    un = copy.copy(hp)
    un.g3, un.c4, un.ws2 = hp.g3_unsplit, P._empty_comb(), hp.ws2_unsplit
    a = run_plan3(hp, L.host, th.host, R.host)
    b = run_plan3(un, L.host, th.host, R.host)
    assert _rel(a, b) <= 1e-13
    t, sgs, _ = hp.g3
    kc = np.concatenate([[0], np.cumsum(sgs["k"].astype(np.int64))])
    work = (kc[t["seg_end"]] - kc[t["seg_begin"]]) * np.minimum(64, t["m"]) * np.minimum(64, t["n"])
    tot = float((work * (-(-t["m"] // 64)) * (-(-t["n"] // 64))).sum())
    assert work.max() <= 2.0 * tot / P.SLOTS


def test_tensor_core_stage3_tile_width():
    """A stage 3 with fewer 128 x 128 tiles than SMs runs 128 x 64 tiles: every output block is
    covered exactly once, and exactly the maps of stage 3's B operands get 64-row boxes."""
    from tnkit_gb300 import workloads
    th, L, W1, W2, R = workloads.mid_bond_problem(device="cpu")
    hp = P.plan_apply(th.layout, L.layout, [(W1.layout, W1.host), (W2.layout, W2.host)], R.layout)
    tc = P.HostPlanTC(hp, th.layout, L.layout, R.layout)
    assert len(P._tiles(tc.t3, tc.s3, P.TC_TILE)) < P.TC_FILL and tc.bn3 == 64
    for k, t in enumerate(tc.t3):
        mine = tc.tiles3[tc.tiles3["task"] == k]
        cells = {(int(a), int(b)) for a, b in zip(mine["m0"], mine["n0"])}
        want = {(a, b) for a in range(0, int(t["m"]), 128) for b in range(0, int(t["n"]), 64)}
        assert cells == want and len(mine) == len(want)
    d = tc.map_desc_box()
    b3 = set(tc.s3["b_map"].tolist())
    for i in range(len(tc.maps)):
        assert d[2 * i, 4] == d[2 * i + 1, 4] == (64 if i in b3 else 128)
    assert np.array_equal(d[:, :4], tc.map_desc())
