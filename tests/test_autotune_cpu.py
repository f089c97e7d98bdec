"""The autotuner's schedules on the CPU: every candidate (split-K on or off at several targets,
tiles in work or sector order) is the same contraction -- the table interpreter gives the
default plan's result for each -- and the shape classes group problems by size."""
import numpy as np
import pytest

from tnkit_gb300 import autotune as AT
from tnkit_gb300 import plan as P
from tnkit_gb300 import workloads
from table_interp import run_plan3


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_every_schedule_computes_the_same_matvec():
    dims = [max(1, d // 3) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=4, device="cpu")
    hp = P.plan_apply(th.layout, L.layout, [(W1.layout, W1.host), (W2.layout, W2.host)],
                      R.layout)
    ref = run_plan3(hp, L.host, th.host, R.host)
    cands = AT.candidates()
    assert len(cands) == 16 and len(AT.candidates(ff=True)) == 8
    labels = set()
    for s in cands:
        sp = AT.scheduled_plan(hp, s)
        got = run_plan3(sp, L.host, th.host, R.host)
        assert _rel(got, ref) <= 1e-13, s
        # the same tiles, possibly reordered; the tasks are the planner's
        assert sorted(map(tuple, sp.g1[2].tolist())) == sorted(map(tuple, hp.g1[2].tolist()))
        if s.split is None:
            assert len(sp.c4[0]) == 0 and sp.ws2 == hp.ws2_unsplit
        labels.add(s.label())
    assert len(labels) == len(cands)


def test_shape_class_groups_by_size():
    def hp_of(scale):
        dims = [max(1, d // scale) for d in workloads.C2_MID_DIMS]
        th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=1, device="cpu")
        return P.plan_apply(th.layout, L.layout, [(W1.layout, W1.host), (W2.layout, W2.host)],
                            R.layout)
    a, b = hp_of(8), hp_of(2)
    assert AT.shape_class(a, False) == AT.shape_class(a, False)
    assert AT.shape_class(a, False) != AT.shape_class(b, False)
    assert AT.shape_class(a, False) != AT.shape_class(a, True)
