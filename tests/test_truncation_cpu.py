"""The truncation's sector scheduling on the CPU: every sector goes to the GPU lane or to one of
the host lanes, longest first, each to the lane that finishes it first; the switches for a host
without its LAPACK thread control and for host-only runs."""
from tnkit_gb300 import linalg as LA

# the charge sectors of a chi=1024 mid-bond two-site block (XXZ N=64)
MID = [(2, 2), (31, 31), (142, 142), (344, 344), (522, 522), (519, 519), (332, 332),
       (128, 128), (26, 26), (2, 2)]


def _cost(lane, n):
    if lane < 0:
        return LA._GPU_MS_PER_ROW * n + 0.4
    return LA._HOST_MS_522 * (n / 522.0) ** 2.1 + 0.05


def test_lanes_cover_every_sector_and_balance_the_largest():
    lanes = LA._assign_sectors(MID, True)
    assert len(lanes) == len(MID)
    assert all(-1 <= l < LA._HOST_LANES for l in lanes)
    # the two ~520-row sectors never share a lane
    big = [lanes[i] for i, s in enumerate(MID) if s[0] > 500]
    assert len(set(big)) == 2
    # the modelled makespan is the largest sector's own cost: nothing queues behind it
    load = {}
    for s, l in zip(MID, lanes):
        load[l] = load.get(l, 0.0) + _cost(l, s[0])
    worst = max(_cost(l, s[0]) for s, l in zip(MID, lanes) if s[0] > 500)
    assert max(load.values()) <= worst + 1e-9


def test_lane_switches():
    assert LA._assign_sectors(MID, False) == [-1] * len(MID)
    host_only = LA._assign_sectors(MID, True, gpu_ok=False)
    assert all(0 <= l < LA._HOST_LANES for l in host_only)
    assert LA._assign_sectors([(40, 40)], True) == [-1]
    assert LA._assign_sectors([(40, 40)], True, gpu_ok=False) == [0]


def test_cut_with_factors_holding_only_the_kept_vectors():
    """The device route hands the cut every sector's full singular values on the host but only
    the kept columns as factors: the cut counts per sector from the full values, as when every
    factor is complete."""
    import numpy as np
    import torch
    from tnkit_gb300.layout import Leg, layout_of
    from tnkit_gb300.tensor import BlockTensor
    a = Leg((-1, 1), (5, 4), 1)
    b = Leg((-1, 1), (6, 4), -1)
    lay = layout_of((a, b), 0)
    m = BlockTensor(lay, torch.zeros(lay.size, dtype=torch.float64))
    blocks = list(LA._blocks(m))
    s = [np.array([0.9, 0.5, 0.3, 0.2, 0.1]), np.array([0.8, 0.6, 0.25, 0.05])]
    chi = 5                      # keeps 0.9, 0.8, 0.6, 0.5, 0.3: three of sector 0, two of 1
    full, part = [], []
    for (_, _, M), sv in zip(blocks, s):
        R, C = M.shape
        k = len(sv)
        U = torch.eye(R, k, dtype=torch.float64)
        Vh = torch.eye(k, C, dtype=torch.float64)
        S = torch.as_tensor(sv)
        full.append((U, S, Vh, sv))
        q = {5: 3, 4: 2}[k]
        part.append((U[:, :q], S[:q], Vh[:q], sv))
    Uf, Sf, Vf, df = LA._trunc_finish(m, blocks, full, chi, "right", True)
    Up, Sp, Vp, dp = LA._trunc_finish(m, blocks, part, chi, "right", True)
    assert Up.layout.legs == Uf.layout.legs and Vp.layout.legs == Vf.layout.legs
    assert torch.equal(Sp, Sf) and torch.equal(Up.data, Uf.data) and torch.equal(Vp.data, Vf.data)
    assert dp == df and abs(df - (0.2 ** 2 + 0.1 ** 2 + 0.25 ** 2 + 0.05 ** 2)) < 1e-15
    assert list(Up.layout.legs[1].dims) == [3, 2]


def _run_tiles(tables, slots, C):
    """Only the listed tiles of each task (64 x 64, clipped), as the grouped GEMM kernel runs
    them; entries outside every tile stay as they were."""
    import numpy as np
    from table_interp import _view
    from tnkit_gb300.plan import TILE_M, TILE_N
    tasks, segs, tiles = tables
    for tl in tiles:
        t = tasks[int(tl["task"])]
        m, n = int(t["m"]), int(t["n"])
        m0, n0 = int(tl["m0"]), int(tl["n0"])
        rows, cols = np.arange(m0, min(m, m0 + TILE_M)), np.arange(n0, min(n, n0 + TILE_N))
        acc = np.zeros((len(rows), len(cols)))
        for s in segs[int(t["seg_begin"]):int(t["seg_end"])]:
            k = int(s["k"])
            A = _view(slots[int(s["a_buf"])], s["a_off"], (m, k), (s["a_rs"], s["a_cs"]))
            B = _view(slots[int(s["b_buf"])], s["b_off"], (k, n), (s["b_rs"], s["b_cs"]))
            acc += float(s["coef"]) * (A[rows] @ B[:, cols])
        C[int(t["c_off"]) + rows[:, None] * int(t["ldc"]) + cols[None, :]] = acc


def test_device_route_product_tables():
    """The device route's grouped-GEMM tables, run tile by tile on the CPU: the Gram matrices'
    tiles cover the triangle the reduction reads (the lower one of the column-major view, G[j n +
    i] for i >= j) with M M^T or M^T M; the other factor is V M or M V^T."""
    import numpy as np
    rng = np.random.default_rng(4)
    shapes = [(70, 90, 1), (130, 40, 2), (5, 3, 1), (64, 64, 2), (200, 129, 1)]
    buf = rng.standard_normal(sum(R * C for R, C, _ in shapes) + 7)
    secs, mo, go = [], 7, 0
    for R, C, side in shapes:
        secs.append((mo, R, C, side, go))
        n = R if side == 1 else C
        mo += R * C
        go += n * n
    G = np.full(go, np.nan)
    _run_tiles(LA._product_tables(LA._gram_products(secs), upper_only=True), [buf], G)
    for (mo, R, C, side, go), _ in zip(secs, shapes):
        M = buf[mo:mo + R * C].reshape(R, C)
        ref = M @ M.T if side == 1 else M.T @ M
        n = ref.shape[0]
        g = G[go:go + n * n]
        lower = np.array([[g[j * n + i] for j in range(i + 1)] for i in range(n)], dtype=object)
        for i in range(n):
            assert np.allclose(np.asarray(lower[i], float), ref[i, :i + 1], rtol=1e-13, atol=1e-12)
    # the other factor
    Z = rng.standard_normal(40000)
    osecs, po = [], 0
    for (mo, R, C, side, _), q in zip(secs, (20, 13, 2, 64, 100)):
        n = R if side == 1 else C
        zo = int(rng.integers(0, 40000 - q * n))
        osecs.append((mo, R, C, side, zo, q, po))
        po += q * (C if side == 1 else R)
    P = np.full(po, np.nan)
    _run_tiles(LA._product_tables(LA._other_products(osecs)), [buf, Z], P)
    for mo, R, C, side, zo, q, po in osecs:
        M = buf[mo:mo + R * C].reshape(R, C)
        n = R if side == 1 else C
        V = Z[zo:zo + q * n].reshape(q, n)
        ref = V @ M if side == 1 else M @ V.T
        assert np.allclose(P[po:po + ref.size].reshape(ref.shape), ref, rtol=1e-13, atol=1e-12)
