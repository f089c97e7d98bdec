"""Batched local problems: many independent two-site H_eff (different chains, bonds, layouts,
MPOs and bond dimensions) applied by one grouped-GEMM launch per stage.

The three-stage tables address every operand by an int64 offset from one of four slot bases
(x0 = L, x1 = theta, x2 = R, workspace) and the output base. K problems become one plan by
placing their operands one after another in arena buffers -- the environments in an L arena and
an R arena, the theta vectors in one batch vector, the intermediates in one workspace -- and
shifting each problem's table offsets by its place in each arena; the tiles of all problems are
then ordered together by decreasing work and stage 3's long tasks split along K over the whole
batch, so small chains fill the SMs that one chain alone leaves idle. The kernels are the
single-problem ones, unchanged: a problem's result is the same contraction, and only the split-K
chunking (hence the order of its partial sums) depends on the batch.

The reference has no batched solve; its oracle is a loop of independent calls, one per chain
(one `apply_two_site`, tnkit/_dmrg.py:162-169, per problem).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from . import ops
from . import plan as P
from .layout import Layout, Leg, layout_of
from .mpo import dense_mpo, to_block_mpo
from .tensor import BlockTensor
from . import workloads



# split-TF32 form of the tensor-core batches: 3 (hi/lo parts staged) or 4 (formed in shared
# memory by the GEMM; the same accuracy)
TC_PASSES = 3

class _Extent:
    """Stand-in output layout of a batched plan: only its size is read."""

    def __init__(self, size: int):
        self.size = int(size)


def _shift_segs(segs: np.ndarray, base: Sequence[int]) -> np.ndarray:
    s = segs.copy()
    b = np.asarray(base, np.int64)
    s["a_off"] += b[s["a_buf"].astype(np.int64)]
    s["b_off"] += b[s["b_buf"].astype(np.int64)]
    return s


def batch_plan(plans: Sequence[P.HostPlan3], bases: Sequence[Sequence[int]],
               out_bases: Sequence[int], ws_total: int, out_total: int,
               kind: str = "apply2-batch") -> P.HostPlan3:
    """One three-stage plan over K problems: problem k's slot-s operand starts at bases[k][s]
    (s = 0, 1, 2 for x0, x1, x2; 3 for its workspace) and its output at out_bases[k]; stage 3
    is split along K over the whole batch."""
    t1s, s1s, t2s, c2s, t3s, s3s = [], [], [], [], [], []
    n1 = n2 = n3 = 0
    macs1 = 0
    for hp, b, ob in zip(plans, bases, out_bases):
        (t1, s1, _), (t2, c2, _), (t3, s3, _) = hp.g1, hp.c2, hp.g3_unsplit
        t = t1.copy()
        t["c_off"] += b[3]
        t["seg_begin"] += n1
        t["seg_end"] += n1
        t1s.append(t)
        s1s.append(_shift_segs(s1, b))
        n1 += len(s1)
        t = t2.copy()
        t["dst_off"] += b[3]
        t["term_begin"] += n2
        t["term_end"] += n2
        t2s.append(t)
        c = c2.copy()
        c["src_off"] += b[3]
        c2s.append(c)
        n2 += len(c2)
        t = t3.copy()
        t["c_off"] += ob
        t["seg_begin"] += n3
        t["seg_end"] += n3
        t3s.append(t)
        s3s.append(_shift_segs(s3, b))
        n3 += len(s3)
        macs1 += hp.macs
    cat = lambda xs, dt: np.concatenate(xs) if xs else np.zeros(0, dt)
    from ._lib import COMB_TASK, COMB_TERM, GEMM_SEG, GEMM_TASK
    return P.HostPlan3(P._GemmArrays(cat(t1s, GEMM_TASK), cat(s1s, GEMM_SEG), macs1),
                       P._CombArrays(cat(t2s, COMB_TASK), cat(c2s, COMB_TERM)),
                       P._GemmArrays(cat(t3s, GEMM_TASK), cat(s3s, GEMM_SEG), 0),
                       ws_total, 0, _Extent(out_total), kind=kind)


Problem = Tuple[Layout, BlockTensor, BlockTensor, BlockTensor, BlockTensor]


class BatchedTwoSiteOperator:
    """H_eff of K independent local problems (theta_layout, L, W1, W2, R) as one operator on the
    concatenation of their theta vectors: `op(x, out)` with x[offsets[k]:offsets[k+1]] problem
    k's theta. The environments are copied once into arena buffers; every call is one launch per
    stage for the whole batch. precision 'f64' (FP64 grouped GEMM), 'ff' (float-float) or 'tc'
    (the tensor-core split-TF32 operator of the same batched plan: operands staged once in FP32,
    one tcgen05 grouped-GEMM launch per GEMM stage for all problems; ~1e-6 relative)."""

    def __init__(self, problems: Sequence[Problem], precision: str = "f64", tune: bool = False,
                 tc_passes: int = TC_PASSES):
        if precision not in ("f64", "ff", "tc"):
            raise ValueError("precision must be 'f64', 'ff' or 'tc'")
        if not problems:
            raise ValueError("no problems")
        dev = problems[0][1].data.device
        if dev.type != "cuda" or any(p[1].data.device != dev or p[4].data.device != dev
                                     for p in problems):
            raise ValueError("all environments must be CUDA tensors on one device")
        self.device = dev
        self.precision = precision
        plans = [ops.host_plan_two_site(th, L, W1, W2, R) for th, L, W1, W2, R in problems]
        sizes = np.array([[L.data.numel(), th.size, R.data.numel(), hp.ws1 + hp.ws2_unsplit]
                          for (th, L, _, _, R), hp in zip(problems, plans)], np.int64)
        starts = np.vstack([np.zeros(4, np.int64), np.cumsum(sizes, 0)])
        self.offsets = starts[:, 1].copy()            # theta / output offsets, K + 1
        self.n = int(starts[-1, 1])
        hp = batch_plan(plans, [tuple(int(v) for v in starts[k]) for k in range(len(plans))],
                        [int(starts[k, 1]) for k in range(len(plans))], int(starts[-1, 3]),
                        self.n)
        self.host = hp
        self.plan = ops.DevicePlan3(hp, dev, ff=precision == "ff")
        self.tc = None
        self.K = len(plans)
        self._owners(plans, starts)
        self.active = np.ones(self.K, bool)
        self._mask_buf = None
        self.macs = hp.macs
        self.ref_macs = sum(P.two_site_ref_macs(th, L.layout, W1.layout, W2.layout, R.layout)
                            for th, L, W1, W2, R in problems)
        self.L = torch.cat([p[1].data.reshape(-1) for p in problems])
        self.R = torch.cat([p[4].data.reshape(-1) for p in problems])
        need = self.plan.ws_elems + (self.plan.out_elems if precision == "ff" else 0)
        self.ws = torch.empty(max(need, 1), dtype=torch.float64, device=dev)
        self.fn = ops._APPLY2["f64" if precision == "tc" else precision]
        self.Lx, self.Rx = self.L, self.R
        if precision == "tc":
            from .mixed import TwoSiteOperatorTC
            self.tc = TwoSiteOperatorTC.from_host_plan(hp, self.L, self.R, self.n,
                                                       passes=tc_passes)
        # the FP64 / float-float launches can drop converged problems' tiles (set_active); the
        # tensor-core operator computes every problem on every call
        self.supports_mask = precision != "tc"
        self.inner, self.tuned = None, None
        if tune and precision != "tc":
            from . import autotune as AT
            xt = torch.randn(self.n, dtype=torch.float64, device=dev)
            yt = torch.empty_like(xt)
            ff = precision == "ff"

            def run(dp):
                w = ops.workspace(dp.ws_elems + (dp.out_elems if ff else 0), dev)
                dp.run(self.fn, self.Lx, xt, self.Rx, yt, w)
            t = AT.tune(hp, run, ff=ff)
            self.host = AT.scheduled_plan(hp, t.schedule)
            self.plan = ops.DevicePlan3(self.host, dev, ff=ff)
            need = self.plan.ws_elems + (self.plan.out_elems if ff else 0)
            self.ws = torch.empty(max(need, 1), dtype=torch.float64, device=dev)
            self._owners(plans, starts)
            self.inner, self.tuned = t.schedule.inner, t
        if precision == "ff":        # float-float copies of the arenas, split once
            lib, sp = _lib.lib(), _lib.stream_ptr()
            self.Lx, self.Rx = torch.empty_like(self.L), torch.empty_like(self.R)
            for src, dst in ((self.L, self.Lx), (self.R, self.Rx)):
                _lib.check(lib.tnk_ff_split(src.data_ptr(), dst.data_ptr(), src.numel(), sp),
                           "ff split")
        self.calls = 0

    def _owners(self, plans, starts):
        """The problem each launch unit (GEMM tile, combination item) belongs to."""
        hp = self.host
        K = len(plans)
        task1 = np.repeat(np.arange(K), [len(p.g1[0]) for p in plans])
        task2 = np.repeat(np.arange(K), [len(p.c2[0]) for p in plans])
        t3, s3, _ = hp.g3
        # an output task by where it writes; a split-K partial (flags bit 4, written to the
        # shared partial region) by where its first K segment reads its Z block
        task3 = np.searchsorted(starts[:, 1], t3["c_off"], side="right") - 1
        part = np.nonzero(t3["flags"] & 16)[0]
        if len(part):
            task3[part] = np.searchsorted(starts[:, 3], s3["a_off"][t3["seg_begin"][part]],
                                          side="right") - 1
        task4 = (np.searchsorted(starts[:, 1], hp.c4[0]["dst_off"], side="right") - 1
                 if len(hp.c4[0]) else np.zeros(0, np.int64))
        self._own = (task1[hp.g1[2]["task"]], task2[hp.c2[2]["task"]],
                     task3[hp.g3[2]["task"]], task4[hp.c4[2]["task"]])

    def set_active(self, mask) -> None:
        """Apply only the problems where `mask` is true from now on: the launch grids (tiles
        and combination items) of the others are dropped; tables and buffers stay. A skipped
        problem's part of the output is left as it was."""
        mask = np.asarray(mask, bool)
        if self.tc is not None:
            raise NotImplementedError("set_active is not available on the tensor-core batch")
        if mask.shape != (self.K,):
            raise ValueError(f"need one flag per problem ({self.K})")
        if np.array_equal(mask, self.active):
            return
        hp = self.host
        units = [hp.g1[2], hp.c2[2], hp.g3[2], hp.c4[2]]
        kept = [u[mask[o]] for u, o in zip(units, self._own)]
        buf, offs = ops._pack(kept, self.device)
        base = buf.data_ptr()
        c = self.plan.c
        c.tiles1, c.n_tiles1 = base + offs[0], len(kept[0])
        c.items2, c.n_items2 = base + offs[1], len(kept[1])
        c.tiles3, c.n_tiles3 = base + offs[2], len(kept[2])
        c.items4, c.n_items4 = base + offs[3], len(kept[3])
        self._mask_buf = buf
        self.active = mask.copy()

    def __call__(self, x: torch.Tensor, out: torch.Tensor = None) -> torch.Tensor:
        if x.numel() != self.n:
            raise ValueError(f"batch vector of {x.numel()} entries, operator takes {self.n}")
        y = torch.empty_like(x) if out is None else out
        if self.tc is not None:
            self.tc(x, y)
        elif self.inner is None:
            self.plan.run(self.fn, self.Lx, x, self.Rx, y, self.ws)
        else:
            lib = _lib.lib()
            prev = lib.tnk_gemm_f64_variant(self.inner)
            try:
                self.plan.run(self.fn, self.Lx, x, self.Rx, y, self.ws)
            finally:
                lib.tnk_gemm_f64_variant(prev)
        self.calls += 1
        return y

    def split(self, x: torch.Tensor) -> List[torch.Tensor]:
        """Views of the K problems' parts of a batch vector."""
        return [x[int(a):int(b)] for a, b in zip(self.offsets[:-1], self.offsets[1:])]


# --------------------------------------------------------------------------------------------
# the batched-solve workload: 64 chains drawn from seed 2
# --------------------------------------------------------------------------------------------


def chain_draws(n_chains: int = 64, seed: int = 2):
    """(model, coupling, N, chi) of each chain: half transverse-field Ising (g uniform in
    [0.5, 1.5], dense), half XXZ (Delta uniform in [0, 2], U(1) blocks), N uniform in
    {16, 24, 32, 48, 64}, chi uniform in {64, 128, 256}, drawn in that order from one numpy
    generator."""
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n_chains):
        model = "tfim" if c < n_chains // 2 else "xxz"
        coupling = float(rng.uniform(0.5, 1.5) if model == "tfim" else rng.uniform(0.0, 2.0))
        N = int(rng.choice([16, 24, 32, 48, 64]))
        chi = int(rng.choice([64, 128, 256]))
        out.append((model, coupling, N, chi))
    return out


def _mid_bond_sectors(N: int, chi: int):
    """S^z sectors of an XXZ chain's mid bond at bond dimension chi: charges of the left half's
    total 2S^z, dimensions in proportion to the square root of their multiplicities (at least
    one state each where kept), summing to min(chi, 2^(N/2))."""
    from math import comb
    h = N // 2
    ks = np.arange(h + 1)
    w = np.sqrt(np.array([comb(h, int(k)) for k in ks], np.float64))
    total = min(chi, 2 ** h)
    d = np.maximum(1, np.floor(w / w.sum() * total)).astype(np.int64)
    while d.sum() > total:
        d[int(np.argmax(d))] -= 1
    while d.sum() < total:
        d[int(np.argmax(w / d))] += 1
    charges = (2 * ks - h).tolist()
    keep = [(int(c), int(x)) for c, x in zip(charges, d) if x > 0]
    return [c for c, _ in keep], [x for _, x in keep]


def chain_problem(model: str, coupling: float, N: int, chi: int, seed: int,
                  device="cuda") -> Problem:
    """A local two-site problem at the mid bond of one chain of the batch: the chain's own bulk
    MPO tensors, seeded random environments and theta with the bond's layout (dense for the
    Ising chain, S^z blocks for XXZ)."""
    rng = np.random.default_rng(seed)
    if model == "tfim":
        Ws = dense_mpo(workloads.tfim_mpo(N, coupling), device=device)
        W1, W2 = Ws[N // 2 - 1], Ws[N // 2]
        D = min(chi, 2 ** (N // 2))
        bond = Leg((0,), (D,), 1)
        phys = W1.legs[2]
    else:
        Wb, _ = to_block_mpo(workloads.xxz_mpo(N, coupling), [[1, -1]] * N, device=device)
        W1, W2 = Wb[N // 2 - 1], Wb[N // 2]
        ch, dims = _mid_bond_sectors(N, chi)
        bond = Leg(tuple(ch), tuple(dims), 1)
        phys = W1.legs[2]
    th = layout_of((bond, phys, phys, bond.flip()), 0)
    Ll = layout_of((bond, W1.legs[0].flip(), bond.flip()), 0)
    Rl = layout_of((bond.flip(), W2.legs[1].flip(), bond), 0)

    def rnd(lay):
        h = rng.standard_normal(lay.size)
        return BlockTensor(lay, torch.as_tensor(h, device=device), h)
    return th, rnd(Ll), W1, W2, rnd(Rl)


def batch_problems(n_chains: int = 64, seed: int = 2, device="cuda") -> List[Problem]:
    """The mid-bond local problems of the batched-solve workload (see chain_draws)."""
    return [chain_problem(m, g, N, chi, seed=1000 + k, device=device)
            for k, (m, g, N, chi) in enumerate(chain_draws(n_chains, seed))]
