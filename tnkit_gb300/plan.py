"""Host planners: block layouts -> task tables of the GB300 kernels.

Every hot-path contraction is planned as three stages over charge blocks (include/tnkit_gb300.h):

  two-site H_eff   Y[p,w,i,j,b] = L[p,w,q] th[q,i,j,b]                         (grouped GEMM)
                   Z[p,s,t,r,b] = sum_{w,i,j} S[w,i,j,s,t,r] Y[p,w,i,j,b]        (combination)
                   out[p,s,t,d] = sum_{r,b} Z[p,s,t,r,b] R[d,r,b]                (grouped GEMM)
  with S = sum_m W1[w,m,s,i] W2[m,r,t,j]; the one-site matvec is the same with one physical leg;
  left env         T[s,d,w,q] = sum_p conj(A[p,s,d]) L[p,w,q]
                   U[d,r,q,y] = sum_{w,s} W[w,r,s,y] T[s,d,w,q]
                   L'[d,r,e]  = sum_{q,y} U[d,r,q,y] A[q,y,e]
  right env        T[u,s,r,y] = sum_x conj(B[u,s,x]) R[x,r,y]
                   V[u,w,p,y] = sum_{r,s} W[w,r,s,p] T[u,s,r,y]
                   R'[u,w,v]  = sum_{p,y} V[u,w,p,y] B[v,p,y]

The intermediates are laid out so that every GEMM operand is a plain strided matrix of one block
(no gathers), the MPO enters only as scalar coefficients of stage 2, and stage 3 sums the charge
sectors of its contraction as K segments of one output tile. These are the contractions of the
reference's tnkit/_dmrg.py:162-231; the planners enumerate the same block pairs its
tnkit/blocks.py:_sym_plan does, from the same canonical layouts.
"""
from __future__ import annotations

import ctypes as C
import itertools
import threading
import math
from collections import defaultdict
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import (COMB_ITEM, COMB_TASK, COMB_TERM, GEMM_SEG, GEMM_TASK, GEMM_TILE)
from .layout import Layout, Leg, canonical

TILE_M = TILE_N = 64          # must match gemm_f64.cu
COMB_CHUNK = 8192             # elements per combination CTA (at least one row)

SLOT_X0, SLOT_X1, SLOT_X2, SLOT_WS = 0, 1, 2, 3


class GemmTable:
    """Tasks and segments of one grouped GEMM stage."""

    def __init__(self):
        self.tasks: List[tuple] = []
        self.segs: List[tuple] = []
        self.macs = 0

    def add(self, c_off, ldc, m, n, segs, accumulate=False):
        b = len(self.segs)
        for s in segs:
            # (a_off, b_off, a_rs, a_cs, b_rs, b_cs, k, a_buf, b_buf, conj, pad, coef)
            self.segs.append(s)
            self.macs += int(m) * int(n) * int(s[6])
        self.tasks.append((c_off, ldc, m, n, b, len(self.segs), 1 if accumulate else 0))

    def arrays(self):
        tasks = np.array(self.tasks, dtype=GEMM_TASK) if self.tasks else np.zeros(0, GEMM_TASK)
        segs = np.array(self.segs, dtype=GEMM_SEG) if self.segs else np.zeros(0, GEMM_SEG)
        return tasks, segs, _tiles_cost(tasks, segs, TILE_M)


def _tiles_cost(tasks, segs, tile):
    """Every (task, m0, n0) tile, ordered by decreasing work (K x tile area), vectorised."""
    if len(tasks) == 0:
        return np.zeros(0, GEMM_TILE)
    m = tasks["m"].astype(np.int64)
    n = tasks["n"].astype(np.int64)
    kcum = np.concatenate([[0], np.cumsum(segs["k"].astype(np.int64))]) if len(segs) else \
        np.zeros(1, np.int64)
    ktot = np.maximum(kcum[tasks["seg_end"]] - kcum[tasks["seg_begin"]], 1)
    tm, tn = -(-m // tile), -(-n // tile)
    cnt = tm * tn
    tid = np.repeat(np.arange(len(tasks)), cnt)
    local = np.arange(int(cnt.sum())) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    m0 = (local // tn[tid]) * tile
    n0 = (local % tn[tid]) * tile
    cost = ktot[tid] * np.minimum(tile, m[tid] - m0) * np.minimum(tile, n[tid] - n0)
    order = np.argsort(-cost, kind="stable")
    tl = np.zeros(len(tid), GEMM_TILE)
    tl["task"], tl["m0"], tl["n0"] = tid[order], m0[order], n0[order]
    return tl


def seg(a_off, a_rs, a_cs, a_buf, b_off, b_rs, b_cs, b_buf, k, coef=1.0, conj=0):
    return (int(a_off), int(b_off), int(a_rs), int(a_cs), int(b_rs), int(b_cs), int(k),
            int(a_buf), int(b_buf), int(conj), 0, float(coef))


class CombTable:
    """Tasks and terms of one combination stage."""

    def __init__(self):
        self.tasks: List[tuple] = []
        self.terms: List[tuple] = []

    def add(self, dst_off, rows, cols, dst_ld, dst_cs, terms):
        b = len(self.terms)
        self.terms.extend(terms)
        self.tasks.append((dst_off, rows, cols, dst_ld, dst_cs, b, len(self.terms)))

    def arrays(self):
        tasks = np.array(self.tasks, dtype=COMB_TASK) if self.tasks else np.zeros(0, COMB_TASK)
        terms = np.array(self.terms, dtype=COMB_TERM) if self.terms else np.zeros(0, COMB_TERM)
        return tasks, terms, _comb_items(tasks)


def _comb_items(tasks) -> np.ndarray:
    """The launch grid of a combination stage: chunks of about COMB_CHUNK elements (at least one
    row) of every task."""
    if not len(tasks):
        return np.zeros(0, COMB_ITEM)
    rows = tasks["rows"].astype(np.int64)
    step = np.maximum(1, COMB_CHUNK // np.maximum(1, tasks["cols"].astype(np.int64)))
    tid, r0, _ = _grid_items(rows, np.ones_like(rows), step, 1)
    it = np.zeros(len(tid), COMB_ITEM)
    it["task"], it["row0"], it["row1"] = tid, r0, np.minimum(rows[tid], r0 + step[tid])
    return it


def term(src_off, src_ld, src_cs, coef):
    return (int(src_off), int(src_ld), int(src_cs), float(coef))


EMPTY_COMB = None


def _empty_comb():
    return (np.zeros(0, COMB_TASK), np.zeros(0, COMB_TERM), np.zeros(0, COMB_ITEM))


SLOTS = 152 * 2            # resident 64x64-tile CTAs of the FP64 / float-float GEMMs


def split_long_tiles(g3, ws_base: int, slots: int = SLOTS, max_chunks: int = 8):
    """Split along K the stage-3 tasks whose tiles are much longer than the average work per
    resident CTA, so one wave of tiles finishes together. Each chunk becomes a task that writes
    its partial product to the workspace (flags bit 4, compact rows at ws_base + ...); stage 4
    sums a split task's partials into its output block in a fixed order. Returns (tables,
    stage-4 tables, workspace elements added). Built by tnk_plan_split_k;
    _split_long_tiles_py states the same in Python."""
    tasks, segs, tiles = g3
    if len(tasks) == 0:
        return g3, _empty_comb(), 0
    tasks, segs = np.ascontiguousarray(tasks), np.ascontiguousarray(segs)
    lib = _lib.lib()
    h = C.c_void_p()
    _lib.check(lib.tnk_plan_split_k(tasks.ctypes.data, len(tasks), segs.ctypes.data,
                                    int(ws_base), slots, max_chunks, TILE_M, TILE_N,
                                    C.byref(h)), "tnk_plan_split_k")
    try:
        (ta, sa, t4, c4), sc = _planb_read(h, [(4, GEMM_TASK), (5, GEMM_SEG), (2, COMB_TASK),
                                               (3, COMB_TERM)])
    finally:
        lib.tnk_planb_free(h)
    if not sc[0]:
        return g3, _empty_comb(), 0
    return (ta, sa, _tiles_cost(ta, sa, TILE_M)), (t4, c4, _comb_items(t4)), sc[1]


def _split_long_tiles_py(g3, ws_base: int, slots: int = SLOTS, max_chunks: int = 8):
    """split_long_tiles in Python (the statement the native planner is tested against)."""
    tasks, segs, tiles = g3
    if len(tasks) == 0:
        return g3, _empty_comb(), 0
    kcum = np.concatenate([[0], np.cumsum(segs["k"].astype(np.int64))])
    ktot = kcum[tasks["seg_end"]] - kcum[tasks["seg_begin"]]
    tile_work = ktot * np.minimum(TILE_M, tasks["m"]) * np.minimum(TILE_N, tasks["n"])
    tm = -(-tasks["m"].astype(np.int64) // TILE_M)
    tn = -(-tasks["n"].astype(np.int64) // TILE_N)
    total = float((tile_work * tm * tn).sum())
    target = max(total / slots, 1.0)
    chunks = np.minimum(np.ceil(tile_work / target).astype(np.int64), max_chunks)
    if (chunks <= 1).all():
        return g3, _empty_comb(), 0
    T, S, red = [], [], CombTable()
    extra = 0
    for ti, t in enumerate(tasks):
        sb, se = int(t["seg_begin"]), int(t["seg_end"])
        c = int(chunks[ti])
        if c <= 1:
            T.append(tuple(t.tolist()[:4]) + (len(S), len(S) + se - sb, int(t["flags"])))
            S.extend(tuple(x.tolist()) for x in segs[sb:se])
            continue
        m, n, K = int(t["m"]), int(t["n"]), int(ktot[ti])
        bounds = [K * j // c for j in range(c + 1)]
        terms = []
        for j in range(c):
            lo, hi = bounds[j], bounds[j + 1]
            part = []
            k0 = 0
            for sg in segs[sb:se]:
                k = int(sg["k"])
                a, b = max(lo, k0), min(hi, k0 + k)
                if a < b:
                    d = a - k0
                    x = list(sg.tolist())
                    x[0] = int(sg["a_off"]) + d * int(sg["a_cs"])
                    x[1] = int(sg["b_off"]) + d * int(sg["b_rs"])
                    x[6] = b - a
                    part.append(tuple(x))
                k0 += k
            off = ws_base + extra
            extra += m * n
            T.append((off, n, m, n, len(S), len(S) + len(part), (int(t["flags"]) & ~1) | 16))
            S.extend(part)
            terms.append(term(off, n, 1, 1.0))
        red.add(int(t["c_off"]), m, n, int(t["ldc"]), 1, terms)
    ta = np.array(T, dtype=GEMM_TASK)
    sa = np.array(S, dtype=GEMM_SEG) if S else np.zeros(0, GEMM_SEG)
    return (ta, sa, _tiles_cost(ta, sa, TILE_M)), red.arrays(), extra


class HostPlan3:
    """A three-stage plan on the host: numpy tables plus sizes and MAC counts (and an optional
    fourth stage summing the split-K partials of stage 3)."""

    def __init__(self, g1: GemmTable, c2: CombTable, g3: GemmTable, ws1, ws2, out_layout,
                 ref_macs=None, kind="", split: bool = True):
        self.g1, self.c2 = g1.arrays(), c2.arrays()
        self.g3_unsplit = g3.arrays()
        self.ws1, self.ws2 = int(ws1), int(ws2)
        self.ws2_unsplit = self.ws2
        if split:
            self.g3, self.c4, extra = split_long_tiles(self.g3_unsplit, self.ws1 + self.ws2)
            self.ws2 += extra
        else:
            self.g3, self.c4 = self.g3_unsplit, _empty_comb()
        self.out_layout = out_layout
        self.macs = g1.macs + g3.macs
        self.comb_terms = len(c2.terms)
        self.ref_macs = ref_macs
        self.kind = kind

    @property
    def ws_elems(self) -> int:
        return self.ws1 + self.ws2


def _check_contract(la: Leg, lb: Leg, what: str):
    if la.charges != lb.charges or la.dims != lb.dims or la.sign != -lb.sign:
        raise ValueError(f"{what}: cannot contract leg {la} with leg {lb}: the sectors must "
                         f"match and the signs be opposite")


def _dense_sector_order(layout: Layout, data: np.ndarray) -> np.ndarray:
    from .layout import to_dense_np
    return to_dense_np(layout, np.asarray(data))


# --------------------------------------------------------------------------- #
# H_eff matvec (one or two sites)
# --------------------------------------------------------------------------- #
_S_CACHE: "OrderedDict" = None
_S_LOCK = threading.Lock()


def _combined_mpo(Ws) -> np.ndarray:
    """Dense combined MPO S[w, i.., s.., r] over sector-ordered indices (S = W1 W2 contracted
    over the middle channel for two sites), cached per pair of MPO tensors: the same site
    tensors recur at every bond of every sweep."""
    global _S_CACHE
    from collections import OrderedDict
    key = tuple((id(l), id(d)) for l, d in Ws)
    with _S_LOCK:
        if _S_CACHE is None:
            _S_CACHE = OrderedDict()
        hit = _S_CACHE.get(key)
        if hit is not None and all(a is l and b is d for (a, b), (l, d) in zip(hit[0], Ws)):
            _S_CACHE.move_to_end(key)
            return hit[1]
    Wd = [_dense_sector_order(l, d) for l, d in Ws]
    if len(Ws) == 1:
        S = np.einsum("wrsi->wisr", Wd[0])
    else:
        S = np.einsum("wmsi,mrtj->wijstr", Wd[0], Wd[1])
    S = np.ascontiguousarray(S, np.float64)
    with _S_LOCK:
        _S_CACHE[key] = (tuple(Ws), S)
        while len(_S_CACHE) > 256:
            _S_CACHE.popitem(last=False)
    return S


def _apply_setup(theta: Layout, L: Layout, Ws: Sequence[Tuple[Layout, np.ndarray]],
                 R: Layout):
    """Checks, the dense combined MPO S[w, in.., out.., r] and the output layout of an H_eff
    plan (shared by the native and the Python planner)."""
    n = len(Ws)
    if n not in (1, 2) or len(theta.legs) != n + 2:
        raise ValueError("plan_apply: one or two sites")
    WL = [w[0] for w in Ws]
    _check_contract(L.legs[2], theta.legs[0], "L.ket/theta.left")
    _check_contract(theta.legs[n + 1], R.legs[2], "theta.right/R.ket")
    _check_contract(L.legs[1], WL[0].legs[0], "L.mpo/W.left")
    _check_contract(WL[-1].legs[1], R.legs[1], "W.right/R.mpo")
    for a in range(n):
        _check_contract(theta.legs[1 + a], WL[a].legs[3], "theta.phys/W.in")
    if n == 2:
        _check_contract(WL[0].legs[1], WL[1].legs[0], "W1.right/W2.left")
    S = _combined_mpo(Ws)
    wleg, rleg = WL[0].legs[0], WL[-1].legs[1]
    ins = [WL[a].legs[3] for a in range(n)]
    outs = [WL[a].legs[2] for a in range(n)]
    wst, rst = wleg.starts(), rleg.starts()
    ist, ost = [l.starts() for l in ins], [l.starts() for l in outs]

    out_legs = (L.legs[0],) + tuple(outs) + (R.legs[0],)
    out = canonical(out_legs, theta.charge)
    return n, S, wleg, rleg, ins, outs, wst, rst, ist, ost, out


def _desc(lay: Layout, keep: list) -> _lib.LayoutDesc:
    k = np.ascontiguousarray(lay.blocks, np.int64)
    sh = np.ascontiguousarray(lay.shapes, np.int64)
    o = np.ascontiguousarray(lay.offsets, np.int64)
    keep.extend((k, sh, o))
    return _lib.LayoutDesc(len(lay.legs), lay.nblocks, k.ctypes.data, sh.ctypes.data,
                           o.ctypes.data)


def _planb_read(h, specs):
    """Copies of the built tables `specs` = [(id, dtype)], then the scalars."""
    lib = _lib.lib()
    out = []
    for tid, dt in specs:
        ptr, cnt = C.c_void_p(), C.c_int64()
        _lib.check(lib.tnk_planb_table(h, tid, C.byref(ptr), C.byref(cnt)), "tnk_planb_table")
        n = int(cnt.value)
        out.append(np.frombuffer((C.c_char * (n * dt.itemsize)).from_address(ptr.value), dt).copy()
                   if n else np.zeros(0, dt))
    sc = (C.c_int64 * 5)()
    _lib.check(lib.tnk_planb_scalars(h, C.cast(sc, C.c_void_p)), "tnk_planb_scalars")
    return out, [int(x) for x in sc]


class _GemmArrays:
    """Ready tables of one grouped-GEMM stage (the native planner's output)."""

    def __init__(self, tasks, segs, macs):
        self.tasks, self.segs, self.macs = tasks, segs, int(macs)

    def arrays(self):
        return self.tasks, self.segs, _tiles_cost(self.tasks, self.segs, TILE_M)


class _CombArrays:
    def __init__(self, tasks, terms):
        self.tasks, self.terms = tasks, terms

    def arrays(self):
        return self.tasks, self.terms, _comb_items(self.tasks)


def plan_apply(theta: Layout, L: Layout, Ws: Sequence[Tuple[Layout, np.ndarray]],
               R: Layout) -> HostPlan3:
    """Plan of (H_eff theta) for n = len(Ws) in {1, 2} sites. `Ws` holds (layout, flat host
    data) of each MPO tensor, legs (wl, wr, s, s'). Built by the native planner
    (tnk_apply_plan_build); _plan_apply_py states the same construction in Python and the tests
    require identical tables."""
    n, S, wleg, rleg, ins, outs, wst, rst, ist, ost, out = _apply_setup(theta, L, Ws, R)
    keep: list = []
    S = np.ascontiguousarray(S, np.float64)
    axes = [wleg] + list(ins) + list(outs) + [rleg]
    starts = np.ascontiguousarray(np.concatenate([l.starts() for l in axes]), np.int64)
    dims = np.ascontiguousarray(np.concatenate([np.asarray(l.dims, np.int64) for l in axes]),
                                np.int64)
    begin = np.concatenate([[0], np.cumsum([len(l.dims) for l in axes])]).astype(np.int64)
    a = _lib.ApplyPlanIn()
    a.n_sites = n
    a.theta, a.L, a.R, a.out = (_desc(theta, keep), _desc(L, keep), _desc(R, keep),
                                _desc(out, keep))
    a.S = S.ctypes.data
    for i, d in enumerate(S.shape):
        a.s_dims[i] = int(d)
    a.sec_start, a.sec_dim = starts.ctypes.data, dims.ctypes.data
    for i, b in enumerate(begin):
        a.sec_begin[i] = int(b)
    lib = _lib.lib()
    h = C.c_void_p()
    _lib.check(lib.tnk_apply_plan_build(C.byref(a), C.byref(h)), "tnk_apply_plan_build")
    try:
        (t1, s1, t2, c2, t3, s3), sc = _planb_read(h, [(0, GEMM_TASK), (1, GEMM_SEG),
                                                       (2, COMB_TASK), (3, COMB_TERM),
                                                       (4, GEMM_TASK), (5, GEMM_SEG)])
    finally:
        lib.tnk_planb_free(h)
    ws1, ws2, macs1, macs3, _ = sc
    return HostPlan3(_GemmArrays(t1, s1, macs1), _CombArrays(t2, c2), _GemmArrays(t3, s3, macs3),
                     ws1, ws2, out, kind=f"apply{n}")


def _plan_apply_py(theta: Layout, L: Layout, Ws: Sequence[Tuple[Layout, np.ndarray]],
                   R: Layout) -> HostPlan3:
    """The construction of plan_apply in Python (the statement the native planner is tested
    against)."""
    n, S, wleg, rleg, ins, outs, wst, rst, ist, ost, out = _apply_setup(theta, L, Ws, R)

    # stage 1 candidates: Y[(p, w, phys.., b)] <- (L block, theta block)
    th_by_q: Dict[int, List[int]] = defaultdict(list)
    for k in range(theta.nblocks):
        th_by_q[int(theta.blocks[k, 0])].append(k)
    ycand: Dict[tuple, Tuple[int, int]] = {}
    y_by_pb: Dict[Tuple[int, int], List[tuple]] = defaultdict(list)
    for kl in range(L.nblocks):
        p, w, q = L.key(kl)
        for kt in th_by_q.get(q, ()):
            tk = theta.key(kt)
            yk = (p, w) + tk[1:]
            ycand[yk] = (kl, kt)
            y_by_pb[(p, tk[-1])].append(yk)

    R_by_d: Dict[int, List[int]] = defaultdict(list)
    for k in range(R.nblocks):
        R_by_d[int(R.blocks[k, 0])].append(k)

    g1, c2, g3 = GemmTable(), CombTable(), GemmTable()
    y_off: Dict[tuple, int] = {}
    ws1 = 0

    def yblock(yk):
        nonlocal ws1
        if yk not in y_off:
            kl, kt = ycand[yk]
            P, Wd_, Q = L.shape(kl)
            tsh = theta.shape(kt)
            ncols = math.prod(tsh[1:])
            y_off[yk] = ws1
            ws1 += P * Wd_ * ncols
            g1.add(y_off[yk], ncols, P * Wd_, ncols,
                   [seg(L.offsets[kl], Q, 1, SLOT_X0, theta.offsets[kt], ncols, 1, SLOT_X1, Q)])
        return y_off[yk]

    zdefs = []      # Z blocks: (key, P, PO, Rd, B, [(y key, coefficient sub-array)], R block)
    tasks3 = []     # (out block, [indices into zdefs])
    for ko in range(out.nblocks):
        ok = out.key(ko)
        p, phys_o, d = ok[0], ok[1:1 + n], ok[-1]
        oshape = out.shape(ko)
        P = oshape[0]
        PO = math.prod(oshape[1:1 + n])
        segs3 = []
        for kr in R_by_d.get(d, ()):
            _, r, b = R.key(kr)
            Rd, B = R.shape(kr)[1], R.shape(kr)[2]
            slices = []
            for yk in y_by_pb.get((p, b), ()):
                w = yk[1]
                phys_i = yk[2:2 + n]
                sub = S[tuple([slice(wst[w], wst[w] + wleg.dims[w])]
                              + [slice(ist[a][phys_i[a]], ist[a][phys_i[a]] + ins[a].dims[phys_i[a]])
                                 for a in range(n)]
                              + [slice(ost[a][phys_o[a]], ost[a][phys_o[a]] + outs[a].dims[phys_o[a]])
                                 for a in range(n)]
                              + [slice(rst[r], rst[r] + Rd)])]
                if sub.any():
                    slices.append((yk, sub))
            if not slices:
                continue
            zdefs.append(((p,) + phys_o + (r, b), P, PO, Rd, B, slices, kr))
            segs3.append(len(zdefs) - 1)
        tasks3.append((ko, segs3))

    # workspace: the Y blocks some Z block uses, then the Z blocks
    for zd in zdefs:
        for yk, _ in zd[5]:
            yblock(yk)
    ws2 = 0
    z_off = []
    for zk, P, PO, Rd, B, slices, kr in zdefs:
        base = ws1 + ws2
        z_off.append(base)
        ws2 += P * PO * Rd * B
        ld = PO * Rd * B
        po_dims = [outs[a].dims[zk[1 + a]] for a in range(n)]
        # per Y block: its nonzero coefficients, flattened as (ww, pi, po, rr) -> value
        prepared = []
        for yk, sub in slices:
            kl, kt = ycand[yk]
            Wd_ = L.shape(kl)[1]
            tsh = theta.shape(kt)
            ncols = math.prod(tsh[1:])
            pi_n = math.prod(tsh[1:1 + n])
            po_n = math.prod(po_dims)
            flat = np.asarray(sub).reshape(Wd_, pi_n, po_n, Rd)
            prepared.append((y_off[yk], Wd_ * ncols, ncols, flat, Wd_, pi_n))
        # one combination task per (phys_o', r') slice of this Z block
        for po_flat in range(math.prod(po_dims)):
            for rr in range(Rd):
                dst = base + (po_flat * Rd + rr) * B
                terms = []
                for yo, src_ld, ncols, flat, Wd_, pi_n in prepared:
                    sub2 = flat[:, :, po_flat, rr]
                    ww_idx, pi_idx = np.nonzero(sub2)
                    for ww, pi in zip(ww_idx.tolist(), pi_idx.tolist()):
                        terms.append((yo + ww * ncols + pi * B, src_ld, 1, float(sub2[ww, pi])))
                c2.add(dst, P, B, ld, 1, terms)
    for ko, segs3 in tasks3:
        oshape = out.shape(ko)
        P, D = oshape[0], oshape[-1]
        PO = math.prod(oshape[1:1 + n])
        segs = []
        for zi in segs3:
            _, _, _, Rd, B, _, kr = zdefs[zi]
            K = Rd * B
            segs.append(seg(z_off[zi], K, 1, SLOT_WS, R.offsets[kr], 1, K, SLOT_X2, K))
        g3.add(out.offsets[ko], D, P * PO, D, segs)
    return HostPlan3(g1, c2, g3, ws1, ws2, out, kind=f"apply{n}")


# --------------------------------------------------------------------------- #
# environment updates
# --------------------------------------------------------------------------- #
def _left_env_setup(L: Layout, A: Layout, W: Tuple[Layout, np.ndarray]):
    WL, wdata = W
    # conj(A) legs carry flipped signs: its left leg meets L's bra leg (same signs as A's)
    _check_contract(A.legs[0].flip(), L.legs[0], "conj(A).left/L.bra")
    _check_contract(L.legs[2], A.legs[0], "L.ket/A.left")
    _check_contract(L.legs[1], WL.legs[0], "L.mpo/W.left")
    _check_contract(A.legs[1].flip(), WL.legs[2], "conj(A).phys/W.out")
    _check_contract(WL.legs[3], A.legs[1], "W.in/A.phys")
    Wd = _dense_sector_order(WL, wdata)          # [w, r, s, y]
    return Wd, canonical((A.legs[2].flip(), WL.legs[1], A.legs[2]), L.charge)


def _right_env_setup(R: Layout, B: Layout, W: Tuple[Layout, np.ndarray]):
    WL, wdata = W
    _check_contract(B.legs[2].flip(), R.legs[0], "conj(B).right/R.bra")
    _check_contract(B.legs[2], R.legs[2], "B.right/R.ket")
    _check_contract(WL.legs[1], R.legs[1], "W.right/R.mpo")
    _check_contract(B.legs[1].flip(), WL.legs[2], "conj(B).phys/W.out")
    _check_contract(WL.legs[3], B.legs[1], "W.in/B.phys")
    Wd = _dense_sector_order(WL, wdata)          # [w, r, s, p]
    return Wd, canonical((B.legs[0].flip(), WL.legs[0], B.legs[0]), R.charge)


def _env_native(side: int, env: Layout, site: Layout, W: Tuple[Layout, np.ndarray],
                kind: str) -> HostPlan3:
    """plan_left_env / plan_right_env by tnk_env_plan_build."""
    Wd, out = (_left_env_setup if side == 0 else _right_env_setup)(env, site, W)
    Wd = np.ascontiguousarray(Wd, np.float64)
    legs = W[0].legs
    keep: list = []
    starts = np.ascontiguousarray(np.concatenate([l.starts() for l in legs]), np.int64)
    dims = np.ascontiguousarray(np.concatenate([np.asarray(l.dims, np.int64) for l in legs]))
    begin = np.concatenate([[0], np.cumsum([len(l.dims) for l in legs])]).astype(np.int64)
    a = _lib.EnvPlanIn()
    a.side = side
    a.env, a.site, a.out = _desc(env, keep), _desc(site, keep), _desc(out, keep)
    a.W = Wd.ctypes.data
    for i, d in enumerate(Wd.shape):
        a.w_dims[i] = int(d)
    a.sec_start, a.sec_dim = starts.ctypes.data, dims.ctypes.data
    for i, b in enumerate(begin):
        a.sec_begin[i] = int(b)
    lib = _lib.lib()
    h = C.c_void_p()
    _lib.check(lib.tnk_env_plan_build(C.byref(a), C.byref(h)), "tnk_env_plan_build")
    try:
        (t1, s1, t2, c2, t3, s3), sc = _planb_read(h, [(0, GEMM_TASK), (1, GEMM_SEG),
                                                       (2, COMB_TASK), (3, COMB_TERM),
                                                       (4, GEMM_TASK), (5, GEMM_SEG)])
    finally:
        lib.tnk_planb_free(h)
    ws1, ws2, macs1, macs3, _ = sc
    return HostPlan3(_GemmArrays(t1, s1, macs1), _CombArrays(t2, c2), _GemmArrays(t3, s3, macs3),
                     ws1, ws2, out, kind=kind)


def plan_left_env(L: Layout, A: Layout, W: Tuple[Layout, np.ndarray]) -> HostPlan3:
    """Plan of L'[d,r,e] = sum L[p,w,q] conj(A[p,s,d]) W[w,r,s,y] A[q,y,e]
    (tnkit/_dmrg.py:216-222). Slots: x0 = A (conjugated), x1 = L, x2 = A. Built by the native
    planner; _plan_left_env_py states the same construction."""
    return _env_native(0, L, A, W, "left_env")


def plan_right_env(R: Layout, B: Layout, W: Tuple[Layout, np.ndarray]) -> HostPlan3:
    """Plan of R'[u,w,v] = sum R[x,r,y] conj(B[u,s,x]) W[w,r,s,p] B[v,p,y]
    (tnkit/_dmrg.py:225-231). Slots: x0 = B (conjugated), x1 = R, x2 = B. Built by the native
    planner; _plan_right_env_py states the same construction."""
    return _env_native(1, R, B, W, "right_env")


def _plan_left_env_py(L: Layout, A: Layout, W: Tuple[Layout, np.ndarray]) -> HostPlan3:
    """plan_left_env in Python (the statement the native planner is tested against)."""
    WL, wdata = W
    Wd, out = _left_env_setup(L, A, W)
    wleg, rleg, sleg, yleg = WL.legs
    wst, rst, sst, yst = (l.starts() for l in WL.legs)

    # stage 1: T[(s,d),(w,q)] per (A block (p,s,d), L block (p,w,q))
    L_by_p: Dict[int, List[int]] = defaultdict(list)
    for k in range(L.nblocks):
        L_by_p[int(L.blocks[k, 0])].append(k)
    tcand = {}
    t_by_dq: Dict[Tuple[int, int], List[tuple]] = defaultdict(list)
    for ka in range(A.nblocks):
        p, s, d = A.key(ka)
        for kl in L_by_p.get(p, ()):
            _, w, q = L.key(kl)
            tk = (s, d, w, q)
            tcand[tk] = (ka, kl)
            t_by_dq[(d, q)].append(tk)
    A_by_e: Dict[int, List[int]] = defaultdict(list)
    for k in range(A.nblocks):
        A_by_e[int(A.blocks[k, 2])].append(k)

    g1, c2, g3 = GemmTable(), CombTable(), GemmTable()
    t_off, ws1 = {}, 0

    def tblock(tk):
        nonlocal ws1
        if tk not in t_off:
            ka, kl = tcand[tk]
            P, S_, D = A.shape(ka)
            _, Wd_, Q = L.shape(kl)
            t_off[tk] = ws1
            ws1 += S_ * D * Wd_ * Q
            g1.add(t_off[tk], Wd_ * Q, S_ * D, Wd_ * Q,
                   [seg(A.offsets[ka], 1, S_ * D, SLOT_X0, L.offsets[kl], Wd_ * Q, 1, SLOT_X1,
                        P, conj=1)])
        return t_off[tk]

    udefs = []     # (key, D, Rd, Q, Y, contributions[(tk, sub W)], kq_e)
    tasks3 = []
    for ko in range(out.nblocks):
        d, r, e = out.key(ko)
        D, Rd, E = out.shape(ko)
        segs3 = []
        for ka2 in A_by_e.get(e, ()):
            q, y, _ = A.key(ka2)
            Q, Yd = A.shape(ka2)[0], A.shape(ka2)[1]
            contrib = []
            for tk in t_by_dq.get((d, q), ()):
                s, _, w, _ = tk
                sub = Wd[wst[w]:wst[w] + wleg.dims[w], rst[r]:rst[r] + Rd,
                         sst[s]:sst[s] + sleg.dims[s], yst[y]:yst[y] + Yd]
                if np.any(sub):
                    contrib.append((tk, sub))
            if not contrib:
                continue
            udefs.append(((d, r, q, y), D, Rd, Q, Yd, contrib, ka2))
            segs3.append(len(udefs) - 1)
        tasks3.append((ko, segs3))
    for ud in udefs:
        for tk, _ in ud[5]:
            tblock(tk)
    ws2, u_off = 0, {}
    for i, (uk, D, Rd, Q, Yd, contrib, ka2) in enumerate(udefs):
        u_off[i] = ws1 + ws2
        ws2 += D * Rd * Q * Yd
        for rr in range(Rd):
            for yy in range(Yd):
                dst = u_off[i] + rr * Q * Yd + yy
                terms = []
                for tk, sub in contrib:
                    ka, kl = tcand[tk]
                    S_, Dd = A.shape(ka)[1], A.shape(ka)[2]
                    Wd_, Qd = L.shape(kl)[1], L.shape(kl)[2]
                    for ww in range(Wd_):
                        for ss in range(S_):
                            c = sub[ww, rr, ss, yy]
                            if c == 0.0:
                                continue
                            src = t_off[tk] + ss * Dd * Wd_ * Qd + ww * Qd
                            terms.append(term(src, Wd_ * Qd, 1, c))
                c2.add(dst, D, Q, Rd * Q * Yd, Yd, terms)
    for ko, segs3 in tasks3:
        D, Rd, E = out.shape(ko)
        segs = []
        for i in segs3:
            _, _, _, Q, Yd, _, ka2 = udefs[i]
            K = Q * Yd
            segs.append(seg(u_off[i], K, 1, SLOT_WS, A.offsets[ka2], E, 1, SLOT_X2, K))
        g3.add(out.offsets[ko], E, D * Rd, E, segs)
    return HostPlan3(g1, c2, g3, ws1, ws2, out, kind="left_env")


def _plan_right_env_py(R: Layout, B: Layout, W: Tuple[Layout, np.ndarray]) -> HostPlan3:
    """plan_right_env in Python (the statement the native planner is tested against)."""
    WL, wdata = W
    Wd, out = _right_env_setup(R, B, W)
    wleg, rleg, sleg, pleg = WL.legs
    wst, rst, sst, pst = (l.starts() for l in WL.legs)

    R_by_x: Dict[int, List[int]] = defaultdict(list)
    for k in range(R.nblocks):
        R_by_x[int(R.blocks[k, 0])].append(k)
    tcand = {}
    t_by_uy: Dict[Tuple[int, int], List[tuple]] = defaultdict(list)
    for kb in range(B.nblocks):
        u, s, x = B.key(kb)
        for kr in R_by_x.get(x, ()):
            _, r, y = R.key(kr)
            tk = (u, s, r, y)
            tcand[tk] = (kb, kr)
            t_by_uy[(u, y)].append(tk)
    B_by_v: Dict[int, List[int]] = defaultdict(list)
    for k in range(B.nblocks):
        B_by_v[int(B.blocks[k, 0])].append(k)

    g1, c2, g3 = GemmTable(), CombTable(), GemmTable()
    t_off, ws1 = {}, 0

    def tblock(tk):
        nonlocal ws1
        if tk not in t_off:
            kb, kr = tcand[tk]
            U, S_, X = B.shape(kb)
            _, Rd, Yd = R.shape(kr)
            t_off[tk] = ws1
            ws1 += U * S_ * Rd * Yd
            g1.add(t_off[tk], Rd * Yd, U * S_, Rd * Yd,
                   [seg(B.offsets[kb], X, 1, SLOT_X0, R.offsets[kr], Rd * Yd, 1, SLOT_X1, X,
                        conj=1)])
        return t_off[tk]

    vdefs, tasks3 = [], []
    for ko in range(out.nblocks):
        u, w, v = out.key(ko)
        U, Wd_, V = out.shape(ko)
        segs3 = []
        for kb2 in B_by_v.get(v, ()):
            _, p, y = B.key(kb2)
            Pd, Yd = B.shape(kb2)[1], B.shape(kb2)[2]
            contrib = []
            for tk in t_by_uy.get((u, y), ()):
                _, s, r, _ = tk
                sub = Wd[wst[w]:wst[w] + Wd_, rst[r]:rst[r] + rleg.dims[r],
                         sst[s]:sst[s] + sleg.dims[s], pst[p]:pst[p] + Pd]
                if np.any(sub):
                    contrib.append((tk, sub))
            if not contrib:
                continue
            vdefs.append(((u, w, p, y), U, Wd_, Pd, Yd, contrib, kb2))
            segs3.append(len(vdefs) - 1)
        tasks3.append((ko, segs3))
    for vd in vdefs:
        for tk, _ in vd[5]:
            tblock(tk)
    ws2, v_off = 0, {}
    for i, (vk, U, Wd_, Pd, Yd, contrib, kb2) in enumerate(vdefs):
        v_off[i] = ws1 + ws2
        ws2 += U * Wd_ * Pd * Yd
        for ww in range(Wd_):
            for pp in range(Pd):
                dst = v_off[i] + (ww * Pd + pp) * Yd
                terms = []
                for tk, sub in contrib:
                    kb, kr = tcand[tk]
                    S_ = B.shape(kb)[1]
                    Rd = R.shape(kr)[1]
                    for ss in range(S_):
                        for rr in range(Rd):
                            c = sub[ww, rr, ss, pp]
                            if c == 0.0:
                                continue
                            src = t_off[tk] + (ss * Rd + rr) * Yd
                            terms.append(term(src, S_ * Rd * Yd, 1, c))
                c2.add(dst, U, Yd, Wd_ * Pd * Yd, 1, terms)
    for ko, segs3 in tasks3:
        U, Wd_, V = out.shape(ko)
        segs = []
        for i in segs3:
            _, _, _, Pd, Yd, _, kb2 = vdefs[i]
            K = Pd * Yd
            segs.append(seg(v_off[i], K, 1, SLOT_WS, B.offsets[kb2], 1, K, SLOT_X2, K))
        g3.add(out.offsets[ko], V, U * Wd_, V, segs)
    return HostPlan3(g1, c2, g3, ws1, ws2, out, kind="right_env")


# --------------------------------------------------------------------------- #
# single-stage plans: tensordot over trailing/leading legs, fuse and split
# --------------------------------------------------------------------------- #
class HostGemmPlan:
    def __init__(self, g: GemmTable, out_layout: Layout):
        self.g = g.arrays()
        self.macs = g.macs
        self.out_layout = out_layout


def plan_tensordot(a: Layout, b: Layout, nc: int) -> HostGemmPlan:
    """out = a . b contracting the last `nc` legs of a with the first `nc` legs of b; output legs
    = free legs of a then free legs of b (tnkit/blocks.py:1156-1192 for this leg order).
    Slots: x0 = a, x1 = b. Built by tnk_tensordot_plan_build; _plan_tensordot_py states the same
    construction."""
    na, nb = len(a.legs), len(b.legs)
    for i in range(nc):
        _check_contract(a.legs[na - nc + i], b.legs[i], "tensordot")
    out = canonical(a.legs[:na - nc] + b.legs[nc:], _add_charge(a.charge, b.charge))
    keep: list = []
    da, db, do = _desc(a, keep), _desc(b, keep), _desc(out, keep)
    lib = _lib.lib()
    h = C.c_void_p()
    _lib.check(lib.tnk_tensordot_plan_build(C.byref(da), C.byref(db), C.byref(do), int(nc),
                                            C.byref(h)), "tnk_tensordot_plan_build")
    try:
        (t, sg), sc = _planb_read(h, [(0, GEMM_TASK), (1, GEMM_SEG)])
    finally:
        lib.tnk_planb_free(h)
    hp = HostGemmPlan.__new__(HostGemmPlan)
    hp.g = (t, sg, _tiles_cost(t, sg, TILE_M))
    hp.macs, hp.out_layout = sc[2], out
    return hp


def _plan_tensordot_py(a: Layout, b: Layout, nc: int) -> HostGemmPlan:
    """plan_tensordot in Python (the statement the native planner is tested against)."""
    na, nb = len(a.legs), len(b.legs)
    for i in range(nc):
        _check_contract(a.legs[na - nc + i], b.legs[i], "tensordot")
    out = canonical(a.legs[:na - nc] + b.legs[nc:], _add_charge(a.charge, b.charge))
    b_by_k: Dict[tuple, List[int]] = defaultdict(list)
    for k in range(b.nblocks):
        b_by_k[b.key(k)[:nc]].append(k)
    a_by_free: Dict[tuple, List[int]] = defaultdict(list)
    for k in range(a.nblocks):
        a_by_free[a.key(k)[:na - nc]].append(k)
    g = GemmTable()
    for ko in range(out.nblocks):
        okey = out.key(ko)
        fa, fb = okey[:na - nc], okey[na - nc:]
        shp = out.shape(ko)
        M = int(np.prod(shp[:na - nc]))
        N = int(np.prod(shp[na - nc:]))
        segs = []
        for ka in a_by_free.get(fa, ()):
            kc = a.key(ka)[na - nc:]
            for kb in b_by_k.get(kc, ()):
                if b.key(kb)[nc:] != fb:
                    continue
                K = int(np.prod(a.shape(ka)[na - nc:]))
                segs.append(seg(a.offsets[ka], K, 1, SLOT_X0, b.offsets[kb], N, 1, SLOT_X1, K))
        g.add(out.offsets[ko], N, M, N, segs)
    return HostGemmPlan(g, out)


def _add_charge(a, b):
    if isinstance(a, tuple):
        return tuple(x + y for x, y in zip(a, b))
    return a + b


class HostCombPlan:
    def __init__(self, c: CombTable, out_layout: Layout, extra=None):
        self.c = c.arrays()
        self.out_layout = out_layout
        self.extra = extra


class FuseInfo:
    """Fused legs of a split of the legs into (rows, cols) at `nrow`: per fused leg the sorted
    signed-total charges and, per fused sector, its sub-sector tuples with row offsets
    (tnkit/blocks.py:1196-1223 for consecutive groups)."""

    def __init__(self, layout: Layout, nrow: int):
        self.layout, self.nrow = layout, nrow
        legs = layout.legs
        groups = (tuple(range(nrow)), tuple(range(nrow, len(legs))))
        self.groups = groups
        self.fused, self.subs = [], []
        for g in groups:
            qs, subs, dims = _fuse_group([legs[a] for a in g])
            self.fused.append(Leg(tuple(qs), tuple(dims), 1))
            self.subs.append(subs)
        self.sector_of = [{t: (k, o, nn) for k, items in enumerate(subs)
                           for t, (o, nn) in items.items()} for subs in self.subs]
        self.matrix = canonical(tuple(self.fused), layout.charge)
        # the same maps as arrays over the flat index of a sector tuple (C order)
        self.nsec = [tuple(len(legs[a].charges) for a in g) for g in groups]
        self.lut = []
        for ns, so in zip(self.nsec, self.sector_of):
            lut = np.zeros((3, int(np.prod(ns)) if ns else 1), np.int64)
            for t, v in so.items():
                lut[:, np.ravel_multi_index(t, ns) if ns else 0] = v
            self.lut.append(lut)

    def lookup(self, g: int, keys: np.ndarray):
        """(fused sector, offset, size) of the sector tuples `keys` (rows) of group g."""
        ns = self.nsec[g]
        flat = np.ravel_multi_index(tuple(np.asarray(keys, np.int64).T), ns) if ns else \
            np.zeros(len(keys), np.int64)
        return self.lut[g][:, flat]


def _fuse_group(legs):
    """The fused leg of consecutive legs: its charges (the signed totals of every sector tuple,
    sorted), per fused sector the sub-sector tuples in product order with their (offset, size),
    and the fused dims. The charge sums and sizes of all tuples are computed at once."""
    n = [len(l.charges) for l in legs]
    if not legs:
        return [0], [{(): (0, 1)}], [1]
    idx = np.indices(n).reshape(len(legs), -1)          # product order (C order)
    q = [l.q * l.sign for l in legs]                      # (sectors, factors)
    tot = sum(qa[ia] for qa, ia in zip(q, idx))           # (tuples, factors)
    size = np.prod([np.asarray(l.dims, np.int64)[ia] for l, ia in zip(legs, idx)], axis=0)
    scalar = not isinstance(legs[0].charges[0], tuple)
    keys = [int(r[0]) for r in tot.tolist()] if scalar else [tuple(r) for r in tot.tolist()]
    by_q: Dict = defaultdict(list)
    tuples = list(map(tuple, idx.T.tolist()))
    for t, k, nn in zip(tuples, keys, size.tolist()):
        by_q[k].append((t, nn))
    qs = sorted(by_q)
    subs, dims = [], []
    for k in qs:
        off, items = 0, {}
        for t, nn in by_q[k]:
            items[t] = (off, nn)
            off += nn
        subs.append(items)
        dims.append(off)
    return qs, subs, dims


def _fuse_group_py(legs):
    """_fuse_group as per-tuple loops (the statement it is tested against)."""
    import itertools
    by_q: Dict = defaultdict(list)
    for t in itertools.product(*(range(len(l.charges)) for l in legs)):
        qv = [np.asarray(l.charges[s]) * l.sign for l, s in zip(legs, t)]
        tot = sum(qv[1:], qv[0])
        key = tuple(int(v) for v in np.ravel(tot)) if np.ndim(tot) else int(tot)
        by_q[key].append(t)
    qs = sorted(by_q)
    subs, dims = [], []
    for q in qs:
        off, items = 0, {}
        for t in by_q[q]:
            nn = int(np.prod([l.dims[s] for l, s in zip(legs, t)]))
            items[t] = (off, nn)
            off += nn
        subs.append(items)
        dims.append(off)
    return qs, subs, dims


def _block_map2(lay: Layout) -> np.ndarray:
    """Block index of every (row sector, column sector) of a two-leg layout, -1 where absent."""
    m = np.full((len(lay.legs[0].charges), len(lay.legs[1].charges)), -1, np.int64)
    if lay.nblocks:
        m[lay.blocks[:, 0], lay.blocks[:, 1]] = np.arange(lay.nblocks)
    return m


def _lookup2(bmap: np.ndarray, i: np.ndarray, j: np.ndarray) -> np.ndarray:
    """bmap[i, j], -1 where (i, j) lies outside it."""
    ok = (i >= 0) & (i < bmap.shape[0]) & (j >= 0) & (j < bmap.shape[1])
    out = np.full(len(i), -1, np.int64)
    out[ok] = bmap[i[ok], j[ok]]
    return out


def _comb_tables(dst, rows, cols, ld, cs, src, src_ld, has):
    """One combination task per entry (with one unit term where `has`, else none)."""
    n = len(dst)
    t = np.zeros(n, COMB_TASK)
    t["dst_off"], t["rows"], t["cols"], t["dst_ld"], t["dst_cs"] = dst, rows, cols, ld, cs
    cnt = np.asarray(has, np.int64)
    end = np.cumsum(cnt)
    t["term_begin"], t["term_end"] = end - cnt, end
    u = np.zeros(int(cnt.sum()), COMB_TERM)
    sel = np.nonzero(cnt)[0]
    u["src_off"], u["src_ld"], u["src_cs"], u["coef"] = src[sel], src_ld[sel], 1, 1.0
    return _CombArrays(t, u)


def plan_fuse(info: FuseInfo) -> HostCombPlan:
    """Copy every block of `info.layout` into its place in the fused matrix (one strided copy
    per block, vectorised; _plan_fuse_py states it block by block)."""
    lay, mat = info.layout, info.matrix
    nr = info.nrow
    if lay.nblocks == 0:
        return HostCombPlan(CombTable(), mat)
    rs, ro, rn = info.lookup(0, lay.blocks[:, :nr])
    cs_, co, cn = info.lookup(1, lay.blocks[:, nr:])
    km = _block_map2(mat)[rs, cs_]
    ncols = mat.shapes[km, 1]
    dst = mat.offsets[km] + ro * ncols + co
    return HostCombPlan(_comb_tables(dst, rn, cn, ncols, 1, lay.offsets, cn,
                                     np.ones(lay.nblocks, bool)), mat)


def _plan_fuse_py(info: FuseInfo) -> HostCombPlan:
    """plan_fuse block by block (the statement the vectorised form is tested against)."""
    lay, mat = info.layout, info.matrix
    c = CombTable()
    nr = info.nrow
    for k in range(lay.nblocks):
        key = lay.key(k)
        r_sec, r_off, r_n = info.sector_of[0][key[:nr]]
        c_sec, c_off, c_n = info.sector_of[1][key[nr:]]
        km = mat.index[(r_sec, c_sec)]
        ncols = mat.shape(km)[1]
        dst = int(mat.offsets[km]) + r_off * ncols + c_off
        c.add(dst, r_n, c_n, ncols, 1, [term(lay.offsets[k], c_n, 1, 1.0)])
    return HostCombPlan(c, mat)


def plan_split_rows(info: FuseInfo, m: Layout) -> HostCombPlan:
    """Split the fused row leg of a matrix layout `m` (legs (F0, k)) back into info's row legs:
    result legs = row legs + (k,). Vectorised; _plan_split_rows_py states it block by block."""
    nr = info.nrow
    rows = info.layout.legs[:nr]
    out = canonical(tuple(rows) + (m.legs[1],), _charge_of_rows(info, m))
    if out.nblocks == 0:
        return HostCombPlan(CombTable(), out)
    rs, ro, rn = info.lookup(0, out.blocks[:, :nr])
    km = _lookup2(_block_map2(m), rs, out.blocks[:, nr])
    ncols = out.shapes[:, -1]
    has = km >= 0
    src = np.where(has, m.offsets[np.maximum(km, 0)] + ro * ncols, 0)
    return HostCombPlan(_comb_tables(out.offsets, rn, ncols, ncols, 1, src, ncols, has), out)


def _plan_split_rows_py(info: FuseInfo, m: Layout) -> HostCombPlan:
    """plan_split_rows block by block (the statement the vectorised form is tested against)."""
    nr = info.nrow
    rows = info.layout.legs[:nr]
    out = canonical(tuple(rows) + (m.legs[1],), _charge_of_rows(info, m))
    c = CombTable()
    for ko in range(out.nblocks):
        key = out.key(ko)
        r_sec, r_off, r_n = info.sector_of[0][key[:nr]]
        km = m.index.get((r_sec, key[nr]))
        ncols = out.shape(ko)[-1]
        if km is None:
            c.add(out.offsets[ko], r_n, ncols, ncols, 1, [])
            continue
        src = int(m.offsets[km]) + r_off * ncols
        c.add(out.offsets[ko], r_n, ncols, ncols, 1, [term(src, ncols, 1, 1.0)])
    return HostCombPlan(c, out)


def _charge_of_rows(info, m):
    return m.charge


def plan_split_cols(info: FuseInfo, m: Layout) -> HostCombPlan:
    """Split the fused column leg of a matrix layout `m` (legs (k, F1)) back into info's column
    legs: result legs = (k,) + col legs. Vectorised; _plan_split_cols_py states it block by
    block."""
    nr = info.nrow
    cols = info.layout.legs[nr:]
    out = canonical((m.legs[0],) + tuple(cols), m.charge)
    if out.nblocks == 0:
        return HostCombPlan(CombTable(), out)
    cs_, co, cn = info.lookup(1, out.blocks[:, 1:])
    km = _lookup2(_block_map2(m), out.blocks[:, 0], cs_)
    nrows = out.shapes[:, 0]
    has = km >= 0
    kk = np.maximum(km, 0)
    src = np.where(has, m.offsets[kk] + co, 0)
    ld = np.where(has, m.shapes[kk, 1], 0)
    return HostCombPlan(_comb_tables(out.offsets, nrows, cn, cn, 1, src, ld, has), out)


def _plan_split_cols_py(info: FuseInfo, m: Layout) -> HostCombPlan:
    """plan_split_cols block by block (the statement the vectorised form is tested against)."""
    nr = info.nrow
    cols = info.layout.legs[nr:]
    out = canonical((m.legs[0],) + tuple(cols), m.charge)
    c = CombTable()
    for ko in range(out.nblocks):
        key = out.key(ko)
        c_sec, c_off, c_n = info.sector_of[1][key[1:]]
        km = m.index.get((key[0], c_sec))
        nrows = out.shape(ko)[0]
        if km is None:
            c.add(out.offsets[ko], nrows, c_n, c_n, 1, [])
            continue
        ld = m.shape(km)[1]
        src = int(m.offsets[km]) + c_off
        c.add(out.offsets[ko], nrows, c_n, c_n, 1, [term(src, ld, 1, 1.0)])
    return HostCombPlan(c, out)


def two_site_ref_macs(theta: Layout, L: Layout, W1: Layout, W2: Layout, R: Layout,
                      parts: bool = False):
    """The reference's algorithmic MAC count of one block `apply_two_site`: the sum over its four
    tensordots of R*K*C per contracted charge (tnkit/blocks.py:1089-1090), i.e. over every
    contributing block pair, |free(a)| * |contracted| * |free(b)|."""
    def tdot(a: Layout, ax_a, b: Layout, ax_b):
        fa = [i for i in range(len(a.legs)) if i not in ax_a]
        fb = [j for j in range(len(b.legs)) if j not in ax_b]
        by = defaultdict(list)
        for kb in range(b.nblocks):
            by[tuple(int(b.blocks[kb, j]) for j in ax_b)].append(kb)
        macs = 0
        outk = set()
        for ka in range(a.nblocks):
            kc = tuple(int(a.blocks[ka, i]) for i in ax_a)
            for kb in by.get(kc, ()):
                macs += int(a.sizes[ka]) * int(np.prod([b.shapes[kb, j] for j in fb]))
                outk.add(tuple(int(a.blocks[ka, i]) for i in fa)
                         + tuple(int(b.blocks[kb, j]) for j in fb))
        legs = tuple(a.legs[i] for i in fa) + tuple(b.legs[j] for j in fb)
        return macs, legs
    m1, l1 = tdot(L, (2,), theta, (0,))            # x1 (p,w,i,j,b)
    x1 = canonical(l1, theta.charge)
    m2, l2 = tdot(W1, (0, 3), x1, (1, 2))          # (m,s,p,j,b)
    x2 = canonical(l2, theta.charge)
    m3, l3 = tdot(W2, (0, 3), x2, (0, 3))          # (r,t,s,p,b) ordering as tensordot yields
    x3 = canonical(l3, theta.charge)
    m4, _ = tdot(R, (1, 2), x3, (0, 4))
    return [m1, m2, m3, m4] if parts else m1 + m2 + m3 + m4


# --------------------------------------------------------------------------- #
# tensor-core (tcgen05, TF32) version of the two-site plan
# --------------------------------------------------------------------------- #
TC_TILE = 128             # must match gemm_tc.cu
TC_FILL = 152             # SMs: a stage with fewer 128 x 128 tiles than this uses 128 x 64
TC_ALIGN = 32             # staged block bases: 32 floats = 128 bytes (TMA needs 16)


def _rup(x: int, a: int) -> int:
    return (int(x) + a - 1) // a * a


def _grid_items(rows, cols, step_r, step_c):
    """(task, r0, c0) of every step_r x step_c cell of each task's rows x cols, task-major, then
    row-major: the enumeration of nested range() loops, vectorised."""
    rows, cols = np.asarray(rows, np.int64), np.asarray(cols, np.int64)
    step_r = np.broadcast_to(np.asarray(step_r, np.int64), rows.shape)
    tr, tc = -(-rows // step_r), -(-cols // step_c)
    cnt = tr * tc
    tid = np.repeat(np.arange(len(rows)), cnt)
    local = np.arange(int(cnt.sum())) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    return tid, (local // tc[tid]) * step_r[tid], (local % tc[tid]) * step_c


def _tiles(tasks, segs, tile, tile_n=None):
    """Every (task, m0, n0) tile of tile x tile_n (default square), ordered by decreasing K
    (stable)."""
    if len(tasks) == 0:
        return np.zeros(0, GEMM_TILE)
    kcum = np.concatenate([[0], np.cumsum(segs["k"].astype(np.int64))]) if len(segs) else \
        np.zeros(1, np.int64)
    ktot = kcum[tasks["seg_end"]] - kcum[tasks["seg_begin"]]
    ktot = np.where(ktot == 0, 1, ktot)
    tid, m0, n0 = _grid_items(tasks["m"], tasks["n"], tile, tile if tile_n is None else tile_n)
    order = np.argsort(-ktot[tid], kind="stable")
    tl = np.zeros(len(tid), GEMM_TILE)
    tl["task"], tl["m0"], tl["n0"] = tid[order], m0[order], n0[order]
    return tl


def _cvt_items(tasks):
    """The 32 x 32 cells of every staging task (rows, cols at positions 2, 3)."""
    from ._lib import CVT_ITEM
    if not len(tasks):
        return np.zeros(0, CVT_ITEM)
    rc = np.array([(t[2], t[3]) for t in tasks], np.int64).reshape(-1, 2)
    tid, r0, c0 = _grid_items(rc[:, 0], rc[:, 1], 32, 32)
    it = np.zeros(len(tid), CVT_ITEM)
    it["task"], it["r0"], it["c0"] = tid, r0, c0
    return it


class HostPlanTC:
    """The two-site plan re-laid out for the tensor cores: every GEMM operand a K-major FP32
    block at a 128-byte-aligned offset of one staging buffer with a 16-byte-multiple row stride
    (theta stored transposed so that it, too, is K-major), tensor-map descriptors of those
    blocks, and the FP64 -> FP32 staging tasks of L, R (once per local problem) and theta (every
    matvec). Derived from the FP64 plan `hp`, whose block structure it keeps."""

    def __init__(self, hp: HostPlan3, theta: Layout, L: Layout, R: Layout, native: bool = True):
        from ._lib import CVT_TASK, TC_SEG
        (t1, s1, _), (t2, c2, i2), (t3, s3, _) = hp.g1, hp.c2, hp.g3_unsplit
        if native:
            self._native(t1, s1, t2, t3, s3)
        else:
            self._python(t1, s1, t2, t3, s3)
        self.tiles1 = _tiles(self.t1, self.s1, TC_TILE)
        self.tiles3 = _tiles(self.t3, self.s3, TC_TILE)
        # stage 3 (few output blocks, long K) in 128 x 64 tiles when its 128 x 128 tiles do not
        # fill the SMs, provided its B operand maps (the staged R blocks) serve no other role:
        # their boxes become 64 rows
        self.bn3 = 128
        b3 = set(self.s3["b_map"].tolist()) if len(self.s3) else set()
        other = set(self.s1["a_map"].tolist()) | set(self.s1["b_map"].tolist()) | \
            set(self.s3["a_map"].tolist())
        if 0 < len(self.tiles3) < TC_FILL and not (b3 & other):
            self.bn3 = 64
            self.tiles3 = _tiles(self.t3, self.s3, TC_TILE, 64)
        self._b3 = b3
        self.c2, self.items2 = c2, i2
        self.cvt_items = {k: _cvt_items(v) for k, v in self.cvt.items()}
        self.stage_elems = _rup(self.cursor, TC_ALIGN)    # hi region; lo at +stage_elems
        self.y32_elems = hp.ws1
        self.out_layout = hp.out_layout
        self.macs = hp.macs

    def _native(self, t1, s1, t2, t3, s3):
        """The tables by tnk_plan_tc_build."""
        from ._lib import CVT_TASK, TC_SEG
        c = lambda a: np.ascontiguousarray(a)
        t1, s1, t2, t3, s3 = c(t1), c(s1), c(t2), c(t3), c(s3)
        lib = _lib.lib()
        h = C.c_void_p()
        _lib.check(lib.tnk_plan_tc_build(t1.ctypes.data, len(t1), s1.ctypes.data, t2.ctypes.data,
                                         len(t2), t3.ctypes.data, len(t3), s3.ctypes.data,
                                         C.byref(h)), "tnk_plan_tc_build")
        maps_dt = np.dtype([("off", "<i8"), ("rows", "<i8"), ("cols", "<i8"), ("ld", "<i8")])
        try:
            (self.t1, self.s1, self.t2, self.t3, self.s3, maps, cl, cr, ct), sc = _planb_read(
                h, [(10, GEMM_TASK), (11, TC_SEG), (12, COMB_TASK), (13, GEMM_TASK),
                    (14, TC_SEG), (15, maps_dt), (16, CVT_TASK), (17, CVT_TASK),
                    (18, CVT_TASK)])
        finally:
            lib.tnk_planb_free(h)
        self.maps = maps.view(np.int64).reshape(-1, 4)
        self.cvt = {"L": cl, "R": cr, "T": ct}
        self.cursor = sc[4]

    def _python(self, t1, s1, t2, t3, s3):
        """The same tables in Python (the statement the native planner is tested against)."""
        from ._lib import CVT_TASK, TC_SEG
        self.cursor = 0
        self.maps: List[tuple] = []
        map_of: Dict[tuple, int] = {}
        cvt = {"L": [], "R": [], "T": []}

        def alloc(n):
            o = self.cursor
            self.cursor += _rup(n, TC_ALIGN)
            return o

        def staged(kind, src_off, rows, cols, transpose=False):
            """Map index of the staged block (source rows x cols at src_off, row-major)."""
            key = (kind, int(src_off))
            if key not in map_of:
                r, c = (cols, rows) if transpose else (rows, cols)
                ld = _rup(c, 4)
                off = alloc(r * ld)
                if kind in cvt:
                    cvt[kind].append((int(src_off), off, rows, cols, cols, ld,
                                      1 if transpose else 0, 0))
                map_of[key] = len(self.maps)
                self.maps.append((off, r, c, ld))
            return map_of[key]

        # stage 1: Y = L theta; A = L block (m x k), B = theta block (k x n) staged as (n x k)
        T1, S1 = [], []
        for t in t1:
            sb, se = int(t["seg_begin"]), int(t["seg_end"])
            segs = []
            for s in s1[sb:se]:
                k = int(s["k"])
                am = staged("L", s["a_off"], int(t["m"]), k)
                bm = staged("T", s["b_off"], k, int(t["n"]), transpose=True)
                segs.append((am, bm, k, 0))
            T1.append((int(t["c_off"]), int(t["ldc"]), int(t["m"]), int(t["n"]), len(S1),
                       len(S1) + len(segs), 0))
            S1.extend(segs)
        # Z blocks (stage-3 A operands) in the staging buffer
        zinfo: Dict[int, tuple] = {}
        for t in t3:
            for s in s3[int(t["seg_begin"]):int(t["seg_end"])]:
                zo = int(s["a_off"])
                if zo not in zinfo:
                    K, M = int(s["k"]), int(t["m"])
                    mi = staged("Z", zo, M, K)
                    zinfo[zo] = (K, M, mi)
        zkeys = np.array(sorted(zinfo), dtype=np.int64)
        # stage 2: remap destinations into the padded Z blocks (sources: Y32 = Y's layout)
        T2 = []
        for t in t2:
            d = int(t["dst_off"])
            j = int(np.searchsorted(zkeys, d, side="right")) - 1
            zo = int(zkeys[j])
            K, M, mi = zinfo[zo]
            off, rows, cols, ld = self.maps[mi]
            rel = d - zo
            row, col = divmod(rel, K)
            if int(t["dst_ld"]) % K:
                raise AssertionError("stage-2 destination stride is not a whole number of rows")
            T2.append((off + row * ld + col, int(t["rows"]), int(t["cols"]),
                       int(t["dst_ld"]) // K * ld, int(t["dst_cs"]), int(t["term_begin"]),
                       int(t["term_end"])))
        # stage 3: out = Z R^T, A = Z block (m x K), B = R block (n x K), FP64 output
        T3, S3 = [], []
        for t in t3:
            segs = []
            for s in s3[int(t["seg_begin"]):int(t["seg_end"])]:
                K = int(s["k"])
                am = zinfo[int(s["a_off"])][2]
                bm = staged("R", s["b_off"], int(t["n"]), K)
                segs.append((am, bm, K, 0))
            T3.append((int(t["c_off"]), int(t["ldc"]), int(t["m"]), int(t["n"]), len(S3),
                       len(S3) + len(segs), 2))
            S3.extend(segs)
        mk = lambda rows, dt: np.array(rows, dtype=dt) if rows else np.zeros(0, dt)
        self.t1, self.s1 = mk(T1, GEMM_TASK), mk(S1, TC_SEG)
        self.t3, self.s3 = mk(T3, GEMM_TASK), mk(S3, TC_SEG)
        self.t2 = mk(T2, COMB_TASK)
        self.cvt = {k: mk(v, CVT_TASK) for k, v in cvt.items()}
        self.maps = np.array(self.maps, np.int64).reshape(-1, 4)

    def map_desc(self) -> np.ndarray:
        """(offset, rows, cols, ld) of every tensor map, hi and lo interleaved."""
        m = np.asarray(self.maps, np.int64).reshape(-1, 4)
        d = np.zeros((2 * len(m), 4), np.int64)
        d[0::2] = m
        d[1::2] = m
        d[1::2, 0] += self.stage_elems
        return d

    def map_desc_box(self) -> np.ndarray:
        """map_desc with a fifth column, the box rows of each map: 64 for stage 3's B operands
        when stage 3 runs 128 x 64 tiles, else 128."""
        d4 = self.map_desc()
        d = np.zeros((len(d4), 5), np.int64)
        d[:, :4] = d4
        d[:, 4] = TC_TILE
        if getattr(self, "bn3", TC_TILE) != TC_TILE and self._b3:
            idx = np.asarray(sorted(self._b3), np.int64)
            d[2 * idx, 4] = self.bn3
            d[2 * idx + 1, 4] = self.bn3
        return d


# --------------------------------------------------------------------------- #
# complex128: the same plans over interleaved (re, im) storage
# --------------------------------------------------------------------------- #
def complexify_gemm(g, tile=TILE_M):
    """A real grouped-GEMM table on complex operands stored as interleaved doubles: each output
    becomes a real-part and an imaginary-part task (output column stride 2, flags bit 2), each
    segment A B the four real products of (Ar + i Ai)(Br + i Bi), with the signs that a
    conjugated operand (segment conj bits) flips."""
    tasks, segs, _ = g
    T, S = [], []
    for t in tasks:
        sb, se = int(t["seg_begin"]), int(t["seg_end"])
        re_segs, im_segs = [], []
        for s in segs[sb:se]:
            ca = -1.0 if int(s["conj"]) & 1 else 1.0
            cb = -1.0 if int(s["conj"]) & 2 else 1.0
            c = float(s["coef"])
            a0, b0 = 2 * int(s["a_off"]), 2 * int(s["b_off"])
            ars, acs, brs, bcs = (2 * int(s["a_rs"]), 2 * int(s["a_cs"]), 2 * int(s["b_rs"]),
                                  2 * int(s["b_cs"]))
            k, abuf, bbuf = int(s["k"]), int(s["a_buf"]), int(s["b_buf"])
            mk = lambda ao, bo, cf: (ao, bo, ars, acs, brs, bcs, k, abuf, bbuf, 0, 0, cf)
            re_segs += [mk(a0, b0, c), mk(a0 + 1, b0 + 1, -c * ca * cb)]
            im_segs += [mk(a0, b0 + 1, c * cb), mk(a0 + 1, b0, c * ca)]
        fl = int(t["flags"]) | 4
        for part, ss in ((0, re_segs), (1, im_segs)):
            T.append((2 * int(t["c_off"]) + part, 2 * int(t["ldc"]), int(t["m"]), int(t["n"]),
                      len(S), len(S) + len(ss), fl))
            S.extend(ss)
    ta = np.array(T, dtype=GEMM_TASK) if T else np.zeros(0, GEMM_TASK)
    sa = np.array(S, dtype=GEMM_SEG) if S else np.zeros(0, GEMM_SEG)
    return ta, sa, _tiles(ta, sa, tile)


def complexify_comb(c):
    """A real combination table (real coefficients) on interleaved complex data: the real and the
    imaginary halves combine separately."""
    tasks, terms, _ = c
    T, U = [], []
    for t in tasks:
        tb, te = int(t["term_begin"]), int(t["term_end"])
        for part in (0, 1):
            b = len(U)
            for u in terms[tb:te]:
                U.append((2 * int(u["src_off"]) + part, 2 * int(u["src_ld"]),
                          2 * int(u["src_cs"]), float(u["coef"])))
            T.append((2 * int(t["dst_off"]) + part, int(t["rows"]), int(t["cols"]),
                      2 * int(t["dst_ld"]), 2 * int(t["dst_cs"]), b, len(U)))
    ct = CombTable()
    ct.tasks, ct.terms = T, U
    return ct.arrays()


class ComplexPlan3:
    """A HostPlan3 for complex128 operands (interleaved storage; workspace in doubles)."""

    def __init__(self, hp: HostPlan3):
        self.g1 = complexify_gemm(hp.g1)
        self.c2 = complexify_comb(hp.c2)
        self.g3 = complexify_gemm(hp.g3)
        self.c4 = complexify_comb(hp.c4)
        self.g3_unsplit = complexify_gemm(hp.g3_unsplit)
        self.ws1, self.ws2 = 2 * hp.ws1, 2 * hp.ws2
        self.out_layout = hp.out_layout
        self.macs = 4 * hp.macs
        self.ref_macs = None
        self.kind = hp.kind + "-c128"

    @property
    def ws_elems(self):
        return self.ws1 + self.ws2
