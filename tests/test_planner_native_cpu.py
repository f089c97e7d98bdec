"""The native host planner (tnk_apply_plan_build, tnk_plan_tc_build) against the planner's
Python statement (plan._plan_apply_py, HostPlanTC(native=False)): identical tables on the
golden local problems (two- and one-site), the chi=1024 mid bond, ragged random U(1) sector
layouts with different left and right bonds, and a U(1) x U(1) Hubbard bond."""
import numpy as np
import pytest

from tnkit_gb300 import plan as P
from tnkit_gb300 import workloads
from tnkit_gb300.layout import Leg, layout_of
from tnkit_gb300.mpo import to_block_mpo
from tnkit_gb300.ops import _host_of


def _lay(meta):
    return layout_of([Leg(tuple(l["charges"]), tuple(l["dims"]), l["sign"]) for l in meta["legs"]],
                     meta["charge"])


def _same_plan(a, b):
    for x, y in zip(a.g1 + a.c2 + a.g3_unsplit + a.g3 + a.c4,
                    b.g1 + b.c2 + b.g3_unsplit + b.g3 + b.c4):
        assert x.dtype == y.dtype and np.array_equal(x, y)
    assert (a.ws1, a.ws2, a.ws2_unsplit, a.macs, a.comb_terms) == \
        (b.ws1, b.ws2, b.ws2_unsplit, b.macs, b.comb_terms)
    assert a.out_layout.legs == b.out_layout.legs and a.kind == b.kind


def _same_tc(hp, th, L, R):
    a = P.HostPlanTC(hp, th, L, R)
    b = P.HostPlanTC(hp, th, L, R, native=False)
    for name in ("t1", "s1", "t2", "t3", "s3", "tiles1", "tiles3"):
        x, y = getattr(a, name), getattr(b, name)
        assert x.dtype == y.dtype and np.array_equal(x, y), name
    assert np.array_equal(a.maps, b.maps) and np.array_equal(a.map_desc(), b.map_desc())
    for k in ("L", "R", "T"):
        assert np.array_equal(a.cvt[k], b.cvt[k]) and np.array_equal(a.cvt_items[k],
                                                                     b.cvt_items[k])
    assert (a.cursor, a.stage_elems, a.y32_elems, a.macs) == \
        (b.cursor, b.stage_elems, b.y32_elems, b.macs)


def _both(th, L, Ws, R, tc=True):
    a = P.plan_apply(th, L, Ws, R)
    b = P._plan_apply_py(th, L, Ws, R)
    _same_plan(a, b)
    if tc and len(Ws) == 2:
        _same_tc(a, th, L, R)
    return a


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_native_planner_golden_problems(golden, tag):
    meta, A = golden
    g = lambda k: (_lay(meta[f"{tag}_{k}"]), A[f"{tag}_{k}"])
    (Ll, _), (Rl, _), (W1l, W1d), (W2l, W2d), (Tl, _) = (g(k) for k in ("L", "R", "W1", "W2",
                                                                       "theta"))
    (Al, _), (R1l, _) = g("A"), g("R1")
    _both(Tl, Ll, [(W1l, W1d), (W2l, W2d)], Rl)
    _both(Al, Ll, [(W1l, W1d)], R1l)


def test_native_planner_chi1024_mid_bond():
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=3, device="cpu")
    hp = _both(th.layout, L.layout, [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))],
               R.layout)
    assert len(hp.c4[0]) > 0          # the split-K stage is exercised too


def _random_bond(rng, charges):
    keep = [c for c in charges if rng.random() < 0.8] or [charges[0]]
    return Leg(tuple(keep), tuple(int(x) for x in rng.integers(1, 40, len(keep))), 1)


@pytest.mark.parametrize("seed", range(8))
def test_native_planner_ragged_u1_layouts(seed):
    """Different, ragged left and right bonds (sectors missing at random) of the XXZ chain."""
    rng = np.random.default_rng(seed)
    Wb, _ = to_block_mpo(workloads.xxz_mpo(6), [[1, -1]] * 6, device="cpu")
    W1, W2 = Wb[2], Wb[3]
    left = _random_bond(rng, list(range(-6, 7, 2)))
    right = _random_bond(rng, list(range(-6, 7, 2)))
    phys = W1.legs[2]
    th = layout_of((left, phys, phys, right.flip()), 0)
    L = layout_of((left, W1.legs[0].flip(), left.flip()), 0)
    R = layout_of((right.flip(), W2.legs[1].flip(), right), 0)
    Ws = [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))]
    if th.nblocks == 0:
        pytest.skip("no allowed theta block for this draw")
    _both(th, L, Ws, R)
    A = layout_of((left, phys, right.flip()), 0)
    R1 = layout_of((right.flip(), W1.legs[1].flip(), right), 0)
    if A.nblocks:
        _both(A, L, [(W1.layout, _host_of(W1))], R1)


def test_native_planner_hubbard_u1xu1_bond():
    """Tuple charges (N_up, N_dn) and the width-6 Jordan-Wigner MPO of the Hubbard chain."""
    rng = np.random.default_rng(4)
    N = 6
    Wb, _ = to_block_mpo(workloads.hubbard_mpo(N, 1.0, 4.0),
                         [workloads.HUBBARD_SITE_CHARGES] * N, device="cpu")
    W1, W2 = Wb[2], Wb[3]
    phys = W1.legs[2]
    ch = [(a, b) for a in range(0, 4) for b in range(0, 4)]
    left = Leg(tuple(ch), tuple(int(x) for x in rng.integers(1, 12, len(ch))), 1)
    ch2 = [(a, b) for a in range(1, 6) for b in range(1, 6)]
    right = Leg(tuple(ch2), tuple(int(x) for x in rng.integers(1, 12, len(ch2))), 1)
    th = layout_of((left, phys, phys, right.flip()), (0, 0))
    L = layout_of((left, W1.legs[0].flip(), left.flip()), (0, 0))
    R = layout_of((right.flip(), W2.legs[1].flip(), right), (0, 0))
    assert th.nblocks > 0
    _both(th, L, [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))], R)


def _same_split(g3, base, **kw):
    a = P.split_long_tiles(g3, base, **kw)
    b = P._split_long_tiles_py(g3, base, **kw)
    for x, y in zip(a[0] + a[1], b[0] + b[1]):
        assert x.dtype == y.dtype and np.array_equal(x, y)
    assert a[2] == b[2]
    return a


def test_native_split_k_matches_python():
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=3, device="cpu")
    hp = P.plan_apply(th.layout, L.layout, [(W1.layout, _host_of(W1)),
                                            (W2.layout, _host_of(W2))], R.layout)
    a = _same_split(hp.g3_unsplit, hp.ws1 + hp.ws2_unsplit)
    assert a[2] > 0 and len(a[1][0]) > 0
    for slots, chunks in ((8, 3), (1000, 8), (2, 1)):
        _same_split(hp.g3_unsplit, 17, slots=slots, max_chunks=chunks)


@pytest.mark.parametrize("seed", range(4))
def test_native_split_k_random_tables(seed):
    from tnkit_gb300._lib import GEMM_SEG, GEMM_TASK
    rng = np.random.default_rng(100 + seed)
    segs, tasks = [], []
    for _ in range(int(rng.integers(1, 30))):
        b = len(segs)
        for _ in range(int(rng.integers(0, 5))):
            segs.append((int(rng.integers(0, 10 ** 6)), int(rng.integers(0, 10 ** 6)),
                         int(rng.integers(1, 500)), 1, 1, int(rng.integers(1, 500)),
                         int(rng.integers(1, 3000)), 3, 2, 0, 0, 1.0))
        tasks.append((int(rng.integers(0, 10 ** 6)), int(rng.integers(1, 500)),
                      int(rng.integers(1, 300)), int(rng.integers(1, 300)), b, len(segs), 0))
    ta, sa = np.array(tasks, GEMM_TASK), np.array(segs, GEMM_SEG)
    g3 = (ta, sa, P._tiles_cost(ta, sa, P.TILE_M))
    _same_split(g3, 5, slots=int(rng.integers(1, 400)), max_chunks=int(rng.integers(1, 9)))


def _both_env(L, A, WA, R, B, WB):
    _same_plan(P.plan_left_env(L, A, WA), P._plan_left_env_py(L, A, WA))
    _same_plan(P.plan_right_env(R, B, WB), P._plan_right_env_py(R, B, WB))


@pytest.mark.parametrize("tag", ["xxz12_b0", "xxz12_b5"])
def test_native_env_planner_golden_problems(golden, tag):
    meta, A = golden
    g = lambda k: (_lay(meta[f"{tag}_{k}"]), A[f"{tag}_{k}"])
    (Ll, _), (Al, _), (W1l, W1d), (Rl, _), (Bl, _), (W2l, W2d) = (
        g(k) for k in ("L", "A", "W1", "R", "B", "W2"))
    _both_env(Ll, Al, (W1l, W1d), Rl, Bl, (W2l, W2d))


def test_native_env_planner_chi1024_mid_bond():
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=3, device="cpu")
    bond, phys = th.layout.legs[0], th.layout.legs[1]
    A = layout_of((bond, phys, bond.flip()), 0)
    _both_env(L.layout, A, (W1.layout, _host_of(W1)), R.layout, A, (W2.layout, _host_of(W2)))


@pytest.mark.parametrize("seed", range(6))
def test_native_env_planner_ragged_u1_layouts(seed):
    rng = np.random.default_rng(200 + seed)
    Wb, _ = to_block_mpo(workloads.xxz_mpo(6), [[1, -1]] * 6, device="cpu")
    W1 = Wb[2]
    left = _random_bond(rng, list(range(-6, 7, 2)))
    right = _random_bond(rng, list(range(-5, 6, 2)))
    phys = W1.legs[2]
    A = layout_of((left, phys, right.flip()), 0)
    if A.nblocks == 0:
        pytest.skip("no allowed block for this draw")
    L = layout_of((left, W1.legs[0].flip(), left.flip()), 0)
    R = layout_of((right.flip(), W1.legs[1].flip(), right), 0)
    Ws = (W1.layout, _host_of(W1))
    _both_env(L, A, Ws, R, A, Ws)


def test_native_env_planner_hubbard():
    rng = np.random.default_rng(6)
    N = 6
    Wb, _ = to_block_mpo(workloads.hubbard_mpo(N, 1.0, 4.0),
                         [workloads.HUBBARD_SITE_CHARGES] * N, device="cpu")
    W1 = Wb[2]
    phys = W1.legs[2]
    ch = [(a, b) for a in range(0, 4) for b in range(0, 4)]
    left = Leg(tuple(ch), tuple(int(x) for x in rng.integers(1, 9, len(ch))), 1)
    ch2 = [(a, b) for a in range(0, 5) for b in range(0, 5)]
    right = Leg(tuple(ch2), tuple(int(x) for x in rng.integers(1, 9, len(ch2))), 1)
    A = layout_of((left, phys, right.flip()), (0, 0))
    L = layout_of((left, W1.legs[0].flip(), left.flip()), (0, 0))
    R = layout_of((right.flip(), W1.legs[1].flip(), right), (0, 0))
    assert A.nblocks > 0
    Ws = (W1.layout, _host_of(W1))
    _both_env(L, A, Ws, R, A, Ws)


def _same_gemm(a, b):
    for x, y in zip(a.g, b.g):
        assert x.dtype == y.dtype and np.array_equal(x, y)
    assert a.macs == b.macs and a.out_layout.legs == b.out_layout.legs


@pytest.mark.parametrize("seed", range(6))
def test_native_tensordot_planner(seed):
    """MPS-site products (one contracted leg) and theta-environment contractions (two legs) on
    ragged U(1) layouts, and a U(1)xU(1) Hubbard pair: identical tables to the Python planner."""
    rng = np.random.default_rng(300 + seed)
    Wb, _ = to_block_mpo(workloads.xxz_mpo(6), [[1, -1]] * 6, device="cpu")
    phys = Wb[2].legs[2]
    a = _random_bond(rng, list(range(-6, 7, 2)))
    b = _random_bond(rng, list(range(-5, 6, 2)))
    c = _random_bond(rng, list(range(-6, 7, 2)))
    A = layout_of((a, phys, b.flip()), 0)
    B2 = layout_of((b, phys, c.flip()), 0)
    if A.nblocks and B2.nblocks:
        _same_gemm(P.plan_tensordot(A, B2, 1), P._plan_tensordot_py(A, B2, 1))
        th = P.plan_tensordot(A, B2, 1).out_layout
        X = layout_of((phys.flip(), c, b.flip()), 0)       # contracts theta's last two legs
        if th.nblocks and X.nblocks:
            _same_gemm(P.plan_tensordot(th, X, 2), P._plan_tensordot_py(th, X, 2))


def test_native_tensordot_planner_hubbard():
    rng = np.random.default_rng(9)
    Wb, _ = to_block_mpo(workloads.hubbard_mpo(6, 1.0, 4.0),
                         [workloads.HUBBARD_SITE_CHARGES] * 6, device="cpu")
    phys = Wb[2].legs[2]
    ch = [(a, b) for a in range(0, 5) for b in range(0, 5)]
    left = Leg(tuple(ch), tuple(int(x) for x in rng.integers(1, 9, len(ch))), 1)
    mid = Leg(tuple(ch), tuple(int(x) for x in rng.integers(1, 9, len(ch))), 1)
    A1 = layout_of((left, phys, mid.flip()), (0, 0))
    A2 = layout_of((mid, phys, left.flip()), (0, 0))
    _same_gemm(P.plan_tensordot(A1, A2, 1), P._plan_tensordot_py(A1, A2, 1))


@pytest.mark.parametrize("seed", range(5))
def test_fuse_group_matches_loops(seed):
    """The fused legs of one, two and three consecutive legs (U(1) and U(1)xU(1) charges, signs
    of both kinds): the same charges, sub-sector offsets and dims as the per-tuple loops."""
    rng = np.random.default_rng(400 + seed)

    def leg(tuple_charges):
        k = int(rng.integers(1, 6))
        if tuple_charges:
            ch = sorted({(int(a), int(b)) for a, b in rng.integers(-3, 4, (k, 2))})
        else:
            ch = sorted({int(a) for a in rng.integers(-6, 7, k)})
        return Leg(tuple(ch), tuple(int(x) for x in rng.integers(1, 9, len(ch))),
                   int(rng.choice([1, -1])))
    for tup in (False, True):
        for nl in (1, 2, 3):
            legs = [leg(tup) for _ in range(nl)]
            assert P._fuse_group(legs) == P._fuse_group_py(legs)


def _same_comb(a, b):
    for x, y in zip(a.c, b.c):
        assert x.dtype == y.dtype and np.array_equal(x, y)
    assert a.out_layout.legs == b.out_layout.legs


def _fuse_cases():
    th, *_ = workloads.mid_bond_problem(seed=3, device="cpu")
    yield th.layout, 0
    rng = np.random.default_rng(10)
    Wb, _ = to_block_mpo(workloads.hubbard_mpo(6, 1.0, 4.0),
                         [workloads.HUBBARD_SITE_CHARGES] * 6, device="cpu")
    phys = Wb[2].legs[2]
    ch = [(a, b) for a in range(0, 5) for b in range(0, 5)]
    left = Leg(tuple(ch), tuple(int(x) for x in rng.integers(1, 9, len(ch))), 1)
    right = Leg(tuple(ch), tuple(int(x) for x in rng.integers(1, 9, len(ch))), 1)
    yield layout_of((left, phys, phys, right.flip()), (0, 0)), (0, 0)


@pytest.mark.parametrize("case", range(2))
def test_vectorised_fuse_and_split_plans(case):
    """The fused matrix copy and both splits back (row side with a truncated bond that keeps
    only some row sectors, column side likewise): identical tables to the block-by-block
    statements."""
    lay, zero = list(_fuse_cases())[case]
    info = P.FuseInfo(lay, 2)
    _same_comb(P.plan_fuse(info), P._plan_fuse_py(info))
    rows, cols = info.matrix.legs
    rng = np.random.default_rng(case)
    keep = sorted(rng.choice(len(rows.charges), max(1, len(rows.charges) // 2), replace=False))
    bond = Leg(tuple(rows.charges[k] for k in keep),
               tuple(int(rng.integers(1, 6)) for _ in keep), 1)
    U = layout_of((rows, bond.flip()), zero)
    Vh = layout_of((bond, cols), lay.charge)
    _same_comb(P.plan_split_rows(info, U), P._plan_split_rows_py(info, U))
    _same_comb(P.plan_split_cols(info, Vh), P._plan_split_cols_py(info, Vh))


def test_native_planners_on_layouts_without_blocks():
    """A theta with no allowed block (bond charges that cannot meet the total charge): every
    planner returns empty tables, identical between the native and Python forms."""
    Wb, _ = to_block_mpo(workloads.xxz_mpo(6), [[1, -1]] * 6, device="cpu")
    W1, W2 = Wb[2], Wb[3]
    phys = W1.legs[2]
    left, right = Leg((-4,), (3,), 1), Leg((4,), (2,), 1)
    th = layout_of((left, phys, phys, right.flip()), 0)
    L = layout_of((left, W1.legs[0].flip(), left.flip()), 0)
    R = layout_of((right.flip(), W2.legs[1].flip(), right), 0)
    assert th.nblocks == 0
    hp = _both(th, L, [(W1.layout, _host_of(W1)), (W2.layout, _host_of(W2))], R)
    assert hp.macs == 0 and len(hp.g1[0]) == 0
    A = layout_of((left, phys, right.flip()), 0)
    _same_plan(P.plan_left_env(L, A, (W1.layout, _host_of(W1))),
               P._plan_left_env_py(L, A, (W1.layout, _host_of(W1))))
    B = layout_of((right, phys, left.flip()), 0)
    _same_gemm(P.plan_tensordot(A, B, 1), P._plan_tensordot_py(A, B, 1))
    info = P.FuseInfo(th, 2)
    _same_comb(P.plan_fuse(info), P._plan_fuse_py(info))
