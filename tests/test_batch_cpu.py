"""Batched local problems on the CPU: the concatenated tables of K independent two-site problems
(dense Ising and U(1) XXZ chains of different sizes), run through the table interpreter, give
each problem's own matvec; the batched-solve workload's draws are reproducible."""
import numpy as np
import pytest

from tnkit_gb300 import batch as B
from tnkit_gb300 import plan as P
from tnkit_gb300.ops import _host_of
from table_interp import run_plan3


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_batched_tables_match_each_problem():
    specs = [("tfim", 0.7, 16, 16), ("xxz", 0.3, 16, 32), ("tfim", 1.3, 24, 32),
             ("xxz", 1.7, 24, 16), ("xxz", 1.0, 32, 24), ("tfim", 1.0, 8, 8)]
    probs = [B.chain_problem(*s, seed=50 + k, device="cpu") for k, s in enumerate(specs)]
    plans = [P.plan_apply(th, L.layout, [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))],
                          R.layout) for th, L, W1, W2, R in probs]
    sizes = np.array([[L.host.size, th.size, R.host.size, hp.ws1 + hp.ws2_unsplit]
                      for (th, L, _, _, R), hp in zip(probs, plans)], np.int64)
    starts = np.vstack([np.zeros(4, np.int64), np.cumsum(sizes, 0)])
    hb = B.batch_plan(plans, [tuple(int(v) for v in starts[k]) for k in range(len(plans))],
                      [int(starts[k, 1]) for k in range(len(plans))], int(starts[-1, 3]),
                      int(starts[-1, 1]))
    rng = np.random.default_rng(3)
    thetas = [rng.standard_normal(th.size) for th, *_ in probs]
    Lcat = np.concatenate([p[1].host for p in probs])
    Rcat = np.concatenate([p[4].host for p in probs])
    got = run_plan3(hb, Lcat, np.concatenate(thetas), Rcat)
    assert hb.macs == sum(hp.macs for hp in plans)
    for k, ((th, L, W1, W2, R), hp) in enumerate(zip(probs, plans)):
        want = run_plan3(hp, L.host, thetas[k], R.host)
        assert _rel(got[starts[k, 1]:starts[k + 1, 1]], want) <= 1e-13


def test_batched_tensor_core_relayout_matches_each_problem():
    """The tensor-core re-layout of a batched plan (staged K-major FP32 blocks of every
    problem's operands in one buffer), interpreted with emulated split TF32, gives each
    problem's own FP64 matvec to split-TF32 accuracy."""
    from table_interp import run_tc_plan
    specs = [("tfim", 0.7, 16, 16), ("xxz", 0.3, 16, 32), ("xxz", 1.0, 24, 24)]
    probs = [B.chain_problem(*s, seed=90 + k, device="cpu") for k, s in enumerate(specs)]
    plans = [P.plan_apply(th, L.layout, [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))],
                          R.layout) for th, L, W1, W2, R in probs]
    sizes = np.array([[L.host.size, th.size, R.host.size, hp.ws1 + hp.ws2_unsplit]
                      for (th, L, _, _, R), hp in zip(probs, plans)], np.int64)
    starts = np.vstack([np.zeros(4, np.int64), np.cumsum(sizes, 0)])
    hb = B.batch_plan(plans, [tuple(int(v) for v in starts[k]) for k in range(len(plans))],
                      [int(starts[k, 1]) for k in range(len(plans))], int(starts[-1, 3]),
                      int(starts[-1, 1]))
    tc = P.HostPlanTC(hb, None, None, None)
    rng = np.random.default_rng(4)
    thetas = [rng.standard_normal(th.size) for th, *_ in probs]
    Lcat = np.concatenate([p[1].host for p in probs])
    Rcat = np.concatenate([p[4].host for p in probs])
    got = run_tc_plan(tc, Lcat, np.concatenate(thetas), Rcat, passes=3)
    for k, ((th, L, W1, W2, R), hp) in enumerate(zip(probs, plans)):
        want = run_plan3(hp, L.host, thetas[k], R.host)
        assert _rel(got[starts[k, 1]:starts[k + 1, 1]], want) <= 2e-5


def test_chain_draws_reproducible():
    d = B.chain_draws(64, 2)
    assert d == B.chain_draws(64, 2) and len(d) == 64
    assert sum(m == "tfim" for m, *_ in d) == 32
    for m, g, N, chi in d:
        assert N in (16, 24, 32, 48, 64) and chi in (64, 128, 256)
        assert (0.5 <= g <= 1.5) if m == "tfim" else (0.0 <= g <= 2.0)


@pytest.mark.parametrize("N,chi", [(16, 64), (16, 256), (64, 256), (8, 1024)])
def test_mid_bond_sectors(N, chi):
    ch, dims = B._mid_bond_sectors(N, chi)
    assert sum(dims) == min(chi, 2 ** (N // 2)) and all(d >= 1 for d in dims)
    assert ch == sorted(ch) and ch == [-c for c in reversed(ch)]


def test_launch_units_owned_by_their_problem():
    """Every tile and combination item of a batched plan maps to the problem whose buffers it
    touches (the basis of dropping converged problems' launch grids)."""
    specs = [("xxz", 1.0, 32, 64), ("tfim", 0.9, 16, 48), ("xxz", 0.4, 24, 32)]
    probs = [B.chain_problem(*s, seed=70 + k, device="cpu") for k, s in enumerate(specs)]
    plans = [P.plan_apply(th, L.layout, [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))],
                          R.layout) for th, L, W1, W2, R in probs]
    sizes = np.array([[L.host.size, th.size, R.host.size, hp.ws1 + hp.ws2_unsplit]
                      for (th, L, _, _, R), hp in zip(probs, plans)], np.int64)
    starts = np.vstack([np.zeros(4, np.int64), np.cumsum(sizes, 0)])
    hb = B.batch_plan(plans, [tuple(int(v) for v in starts[k]) for k in range(3)],
                      [int(starts[k, 1]) for k in range(3)], int(starts[-1, 3]),
                      int(starts[-1, 1]))
    op = B.BatchedTwoSiteOperator.__new__(B.BatchedTwoSiteOperator)
    op.host = hb
    op._owners(plans, starts)
    own1, own2, own3, own4 = op._own
    t1, s1, tl1 = hb.g1
    assert np.array_equal(own1, np.searchsorted(starts[:, 3], t1["c_off"][tl1["task"]],
                                                side="right") - 1)
    t3, s3, tl3 = hb.g3
    for o, t in zip(own3, tl3["task"]):
        sb, se = int(t3["seg_begin"][t]), int(t3["seg_end"][t])
        assert ((s3["b_off"][sb:se] >= starts[o, 2]) & (s3["b_off"][sb:se] < starts[o + 1, 2])).all()
    t4 = hb.c4[0]
    if len(t4):
        assert np.array_equal(own4, np.searchsorted(starts[:, 1], t4["dst_off"][hb.c4[2]["task"]],
                                                    side="right") - 1)
    assert len(own2) == len(hb.c2[2]) and own2.max() == 2


def test_full_64_chain_workload_plans():
    """Every local problem of the 64-chain batch workload plans, and the concatenated plan of all
    64 has every problem's tasks, segments, combination terms and MAC count."""
    probs = B.batch_problems(64, seed=2, device="cpu")
    plans = [P.plan_apply(th, L.layout, [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))],
                          R.layout) for th, L, W1, W2, R in probs]
    sizes = np.array([[L.host.size, th.size, R.host.size, hp.ws1 + hp.ws2_unsplit]
                      for (th, L, _, _, R), hp in zip(probs, plans)], np.int64)
    starts = np.vstack([np.zeros(4, np.int64), np.cumsum(sizes, 0)])
    hb = B.batch_plan(plans, [tuple(int(v) for v in starts[k]) for k in range(64)],
                      [int(starts[k, 1]) for k in range(64)], int(starts[-1, 3]),
                      int(starts[-1, 1]))
    assert len(hb.g1[0]) == sum(len(p.g1[0]) for p in plans)
    assert len(hb.c2[1]) == sum(len(p.c2[1]) for p in plans)
    assert len(hb.g3_unsplit[1]) == sum(len(p.g3_unsplit[1]) for p in plans)
    assert hb.macs == sum(p.macs for p in plans)
    assert int(starts[-1, 1]) == sum(th.size for th, *_ in probs)
