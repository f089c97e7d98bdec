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
