"""Autotuning of the three-stage grouped-GEMM schedule on the problem at hand.

A three-stage plan fixes what is computed; how its tiles are scheduled is free. The tuner
times, with CUDA events on the launching stream, every combination of

  inner    the FP64 grouped GEMM's inner product: per-thread FMA tiles or DMMA (mma.sync
           m8n8k4) tiles (tnk_gemm_f64_variant); float-float plans have one
  split    stage 3's split-K schedule: off, or split_long_tiles with the average work of
           SLOTS / 2, SLOTS, 2 SLOTS resident tiles as the target (max 8 chunks per task)
  order    the launch order of the tiles of both GEMM stages: decreasing work (the planner's
           default, long tasks first) or task order (the plan's own sector order)

on the caller's operands, and keeps the fastest. The results are identical up to the order of
partial sums (split-K) -- the tuner never changes the arithmetic. A choice is cached per shape
class (the plan's kind, tile count and K depth rounded to powers of two), so the many local
problems of a sweep that share a class are tuned once.

The reference has no schedule to tune (it calls one library GEMM per sector, tnkit/blocks.py:
1185-1191); this is the schedule tuner of the batched-solve configuration.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
import torch

from . import _lib
from . import plan as P


@dataclass(frozen=True)
class Schedule:
    inner: int = 0                   # 0: FMA tile, 1: DMMA tile
    split: Optional[int] = P.SLOTS   # split-K target slots, None: no split
    order: str = "work"              # 'work' (decreasing work) or 'task' (sector order)

    def label(self) -> str:
        return (f"{'dmma' if self.inner else 'fma'}/"
                f"{'nosplit' if self.split is None else f'split{self.split}'}/{self.order}")


DEFAULT = Schedule()


@dataclass
class Tuned:
    schedule: Schedule
    ms: float
    table: Dict[str, float] = field(default_factory=dict)


_CACHE: Dict[tuple, Tuned] = {}


def _task_order(tiles: np.ndarray) -> np.ndarray:
    if len(tiles) == 0:
        return tiles
    return tiles[np.lexsort((tiles["n0"], tiles["m0"], tiles["task"]))]


def scheduled_plan(hp: P.HostPlan3, s: Schedule) -> P.HostPlan3:
    """`hp` with schedule `s`'s stage-3 split and tile order (same tasks and results)."""
    out = copy.copy(hp)
    if s.split is None:
        out.g3, out.c4, extra = hp.g3_unsplit, P._empty_comb(), 0
    else:
        out.g3, out.c4, extra = P.split_long_tiles(hp.g3_unsplit, hp.ws1 + hp.ws2_unsplit,
                                                   slots=s.split)
    out.ws2 = hp.ws2_unsplit + extra
    if s.order == "task":
        t1, s1, l1 = out.g1
        t3, s3, l3 = out.g3
        out.g1 = (t1, s1, _task_order(l1))
        out.g3 = (t3, s3, _task_order(l3))
    return out


def candidates(ff: bool = False) -> List[Schedule]:
    inner = (0,) if ff else (0, 1)
    splits = (None, P.SLOTS // 2, P.SLOTS, 2 * P.SLOTS)
    return [Schedule(i, sp, o) for i in inner for sp in splits for o in ("work", "task")]


def shape_class(hp: P.HostPlan3, ff: bool) -> tuple:
    t3, s3, _ = hp.g3_unsplit
    kmax = int(s3["k"].max()) if len(s3) else 0
    b = lambda v: int(round(math.log2(max(int(v), 1))))
    return (hp.kind, ff, b(len(hp.g1[2]) + len(hp.g3_unsplit[2])), b(kmax), b(hp.macs))


def tune(hp: P.HostPlan3, run: Callable[[object], None], ff: bool = False, reps: int = 3,
         key: Optional[tuple] = None, cands: Optional[List[Schedule]] = None) -> Tuned:
    """The fastest schedule of `hp`: `run(device_plan)` applies the plan once to the caller's
    operands (on the current stream); each candidate runs once untimed, then `reps` times
    between CUDA events, with the inner-product variant set around it. Cached under `key`
    (default: the shape class)."""
    from .ops import DevicePlan3
    key = key if key is not None else shape_class(hp, ff)
    if key in _CACHE:
        return _CACHE[key]
    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    prev = lib.tnk_gemm_f64_variant(-1)
    table, best = {}, None
    try:
        for s in (cands or candidates(ff)):
            dp = DevicePlan3(scheduled_plan(hp, s), dev, ff=ff)
            lib.tnk_gemm_f64_variant(s.inner)
            run(dp)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                run(dp)
            b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b) / reps
            table[s.label()] = ms
            if best is None or ms < best[1]:
                best = (s, ms)
    finally:
        lib.tnk_gemm_f64_variant(prev)
    res = Tuned(best[0], best[1], table)
    _CACHE[key] = res
    return res


def clear_cache() -> None:
    _CACHE.clear()
