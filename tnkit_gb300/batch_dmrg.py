"""Lockstep DMRG of many independent chains: every round, each chain that still has a bond to
solve in its sweeps contributes that bond's local problem; the problems are applied together by
one batched plan (`batch.BatchedTwoSiteOperator`: one launch per stage for all chains) inside a
batched thick-restart Lanczos, then each chain truncates and updates its environment.

Batched Lanczos. The K local problems are K independent Krylov recurrences over one
concatenated basis (row j holds every chain's j-th basis vector, chain k at columns
[offsets[k], offsets[k+1])). All chains take one matvec per iteration, so their basis indices
and restarts stay in step. Every vector operation is per chain: the fused Gram-Schmidt passes
(tnk_cgs_pass_f64) run on each chain's segment of the basis -- a row stride equal to the batch
length -- so the reductions never mix chains; the K projected problems are diagonalised
together (numpy's batched symmetric eigensolver). A chain stops at its own Ritz residual or
breakdown (the reference's rules, tnkit/eigensolver.py:611-623); its segment is then left
alone while the others continue. The algorithm per chain is `lanczos_ground_restart`'s.

The reference has no batched solver; its oracle is a loop of independent `dmrg` calls, one per
chain (tnkit/_dmrg.py:439-522).
"""
from __future__ import annotations

import time
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from . import linalg as LA
from . import ops
from .batch import BatchedTwoSiteOperator
from .dmrg import _resolve, setup_chain
from .tensor import BlockTensor

_MAXNV = 64
_REC = 1 + 2 * _MAXNV            # per chain: beta, c1[0:64], c2[0:64]
_SUB, _DOT, _NRM = 1, 2, 4


class _Segments:
    """The Lanczos vector kernels on the chains' segments of a batch vector: per chain
    (`cgs2`, `nrm2`, `scale_div`: one launch per chain each) or, with `segmented`, every listed
    chain in one launch per pass (`cgs2_all`, `nrm2_all`, `scale_div_all`:
    tnk_cgs_pass_seg_f64 / tnk_scale_div_seg_f64, grid rows = chains)."""

    def __init__(self, offsets: Sequence[int], n: int, device, segmented: bool = True):
        self.off = [int(x) for x in offsets]
        self.K = len(self.off) - 1
        self.n = int(n)
        self.lib = _lib.lib()
        self.sp = _lib.stream_ptr()
        self.red = torch.empty(_lib.TNK_RED_ELEMS, dtype=torch.float64, device=device)
        self.cnt = torch.zeros(max(4, self.K), dtype=torch.int32, device=device)
        self.rec = torch.zeros((self.K, _REC), dtype=torch.float64, device=device)
        self.hrec = torch.zeros((self.K, _REC), dtype=torch.float64, pin_memory=True)
        self.segmented = segmented
        self.off_dev = torch.as_tensor(np.asarray(self.off, np.int64), device=device)
        self.lens = np.diff(np.asarray(self.off, np.int64))
        self._ids_key, self._ids = None, None
        self.device = device

    def ids(self, act):
        """Device int32 list of the chains `act` (uploaded when the set changes)."""
        key = tuple(int(c) for c in act)
        if key != self._ids_key:
            self._ids = torch.as_tensor(np.asarray(key, np.int32), device=self.device)
            self._ids_key = key
        return self._ids

    def _seg_pass(self, V, nv, w, act, cin_slot, out_slot, mode):
        ids = self.ids(act)
        rec = self.rec.data_ptr()
        cin = None if cin_slot is None else rec + 8 * cin_slot
        _lib.check(self.lib.tnk_cgs_pass_seg_f64(
            None if V is None else V.data_ptr(), self.n, nv, cin, w.data_ptr(),
            self.off_dev.data_ptr(), ids.data_ptr(), len(act), int(self.lens[list(act)].max()),
            _REC, rec + 8 * out_slot, mode, self.red.data_ptr(), self.cnt.data_ptr(), self.sp),
            "cgs_pass_seg")

    def cgs2_all(self, V, nv, w, act):
        """cgs2 of every chain in `act`, three launches in all."""
        self._seg_pass(V, nv, w, act, None, 1, _DOT)
        self._seg_pass(V, nv, w, act, 1, 1 + _MAXNV, _SUB | _DOT)
        self._seg_pass(V, nv, w, act, 1 + _MAXNV, 0, _SUB | _NRM)

    def nrm2_all(self, x, act):
        self._seg_pass(None, 0, x, act, None, 0, _NRM)

    def scale_div_all(self, x, y, act):
        """y_c = x_c / beta_c for every chain in `act`, one launch."""
        ids = self.ids(act)
        _lib.check(self.lib.tnk_scale_div_seg_f64(
            x.data_ptr(), y.data_ptr(), self.off_dev.data_ptr(), ids.data_ptr(), len(act),
            int(self.lens[list(act)].max()), self.rec.data_ptr(), _REC, 1.0, self.sp),
            "scale_div_seg")

    def seg(self, k):
        k = int(k)
        return self.off[k], self.off[k + 1] - self.off[k]

    def raddr(self, k, i):
        return int(self.rec.data_ptr() + 8 * (int(k) * _REC + int(i)))

    def cgs(self, V: torch.Tensor, nv: int, w: torch.Tensor, k: int, cin, out, mode):
        a, nk = self.seg(k)
        _lib.check(self.lib.tnk_cgs_pass_f64(V.data_ptr() + 8 * a, V.stride(0), nv, cin,
                                             w.data_ptr() + 8 * a, nk, out, mode,
                                             self.red.data_ptr(), self.cnt.data_ptr(),
                                             self.sp), "cgs_pass")

    def cgs2(self, V, nv, w, k):
        """c1 = V^T w; w -= V c1, c2 = V^T w; w -= V c2, beta = ||w|| on chain k's segment."""
        c1, c2 = self.raddr(k, 1), self.raddr(k, 1 + _MAXNV)
        self.cgs(V, nv, w, k, None, c1, _DOT)
        self.cgs(V, nv, w, k, c1, c2, _SUB | _DOT)
        self.cgs(V, nv, w, k, c2, self.raddr(k, 0), _SUB | _NRM)

    def nrm2(self, x, k):
        a, nk = self.seg(k)
        _lib.check(self.lib.tnk_nrm2_f64(x.data_ptr() + 8 * a, nk, self.raddr(k, 0),
                                         self.red.data_ptr(), self.sp), "nrm2")

    def scale_div(self, x, y, k):
        """y_k = x_k / beta_k (beta from chain k's record slot 0)."""
        a, nk = self.seg(k)
        _lib.check(self.lib.tnk_scale_div_f64(x.data_ptr() + 8 * a, y.data_ptr() + 8 * a, nk,
                                              self.raddr(k, 0), 1.0, self.sp), "scale_div")

    def read(self) -> np.ndarray:
        self.hrec.copy_(self.rec, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return self.hrec.numpy()


def lanczos_ground_batched(op, x0: torch.Tensor, offsets: Sequence[int], tol: float = 1e-9,
                           max_iter: int = 200, m: int = 40, k: int = 10,
                           segmented: bool = True):
    """Lowest eigenpair of each of K symmetric operators applied together by `op(x, out)` on
    the concatenation of their vectors (chain c at [offsets[c], offsets[c+1])), from the start
    x0. With `segmented` every Gram-Schmidt pass and normalisation is one launch for all active
    chains, else one launch per chain. Returns (E (K,), X (the K unit Ritz vectors,
    concatenated), info)."""
    if m + 1 > _MAXNV or m < 2 or not 0 < k < m:
        raise ValueError(f"need 0 < k < m <= {_MAXNV - 1}")
    dev = x0.device
    n = x0.numel()
    S = _Segments(offsets, n, dev, segmented)
    K = S.K
    Vb = torch.empty((m + 1, n), dtype=torch.float64, device=dev)
    w = torch.empty(n, dtype=torch.float64, device=dev)
    X = torch.zeros(n, dtype=torch.float64, device=dev)
    E = np.full(K, np.nan)
    iters = np.zeros(K, np.int64)
    conv = np.zeros(K, bool)
    if segmented:
        S.nrm2_all(x0, list(range(K)))
    else:
        for c in range(K):
            S.nrm2(x0, c)
    nrm0 = S.read()[:, 0].copy()
    active = np.isfinite(nrm0) & (nrm0 > 1e-300)
    if segmented:
        if active.any():
            S.scale_div_all(x0, Vb[0], np.nonzero(active)[0])
    else:
        for c in np.nonzero(active)[0]:
            S.scale_div(x0, Vb[0], c)
    T = np.zeros((K, m + 1, m + 1))
    j, it, restarts = 0, 0, 0
    while active.any():
        op(Vb[j], w)
        act = np.nonzero(active)[0]
        if segmented:
            S.cgs2_all(Vb, j + 1, w, act)
        else:
            for c in act:
                S.cgs2(Vb, j + 1, w, c)
        h = S.read()
        alpha, beta = h[:, 1 + j].copy(), h[:, 0].copy()
        T[act, j, j] = alpha[act]
        cur = j + 1
        it += 1
        if cur == 1:
            ev, evec = alpha[act][:, None], np.ones((len(act), 1, 1))
        else:
            ev, evec = np.linalg.eigh(T[act, :cur, :cur])
        y = evec[:, :, 0]
        res = np.abs(beta[act] * y[:, cur - 1])
        brk = (~np.isfinite(beta[act]) | ~np.isfinite(alpha[act])
               | (beta[act] < 1e-12 * np.maximum(1.0, np.abs(alpha[act]))))
        done = brk | (res < tol) | (it >= max_iter)
        iters[act] = it
        for q in np.nonzero(done)[0]:
            c = act[q]
            a, nk = S.seg(c)
            E[c] = ev[q, 0]
            conv[c] = bool(brk[q] or res[q] < tol)
            yq = torch.as_tensor(np.ascontiguousarray(y[q]), device=dev)
            torch.mv(Vb[:cur, a:a + nk].t(), yq, out=X[a:a + nk])
            active[c] = False
        keep = np.nonzero(~done)[0]
        if len(keep) == 0:
            break
        if done.any() and getattr(op, "supports_mask", False):
            op.set_active(active)                     # converged chains leave the launches
        if cur >= m:                                  # thick restart, all chains in step
            kk = min(k, cur - 1)
            for q in keep:
                c = act[q]
                a, nk = S.seg(c)
                Yk = torch.as_tensor(np.ascontiguousarray(evec[q][:, :kk].T), device=dev)
                Vb[:kk, a:a + nk].copy_(torch.mm(Yk, Vb[:cur, a:a + nk]))
                border = beta[c] * evec[q][cur - 1, :kk]
                T[c] = 0.0
                T[c, np.arange(kk), np.arange(kk)] = ev[q, :kk]
                T[c, :kk, kk] = border
                T[c, kk, :kk] = border
                if not segmented:
                    S.scale_div(w, Vb[kk], c)
            if segmented:
                S.scale_div_all(w, Vb[kk], act[keep])
            j = kk
            restarts += 1
        else:
            for q in keep:
                c = act[q]
                T[c, j, j + 1] = T[c, j + 1, j] = beta[c]
                if not segmented:
                    S.scale_div(w, Vb[j + 1], c)
            if segmented:
                S.scale_div_all(w, Vb[j + 1], act[keep])
            j += 1
    torch.cuda.current_stream().synchronize()
    return E, X, {"iters": iters, "converged": conv, "restarts": restarts, "matvecs": it}


def dmrg_batch(mpos: Sequence, chis: Sequence[int], charges: Optional[Sequence] = None,
               seeds: Optional[Sequence[int]] = None, options=None, pipeline: bool = False,
               **kw):
    """Two-site DMRG of K independent chains (MPOs of any lengths, block or dense, their own
    bond dimensions, charges and seeds) in lockstep rounds: round r solves bond step r of every
    chain that has one (a sweep is N-1 bonds left to right, then N-1 right to left), all local
    problems in one batched Lanczos on one batched plan; truncation and the environment update
    stay per chain. Options as `dmrg` (n_sweeps, eig_tol, restart_m, restart_k, max_iter,
    svd_method, svd_driver, device; precision 'f64' or 'ff' for the batched matvec, or 'mixed' /
    'mixed-ff': each round's problems first solved together on the tensor cores to mixed_tol_lo,
    then polished in FP64 / float-float; no convergence stop: every chain runs n_sweeps). With `pipeline` the chains run as two groups
    whose eigensolver and truncation phases overlap (the results are the same; measured on
    GB300 it gains ~3 %: both phases need the FP64 units and the host cores). Returns
    (energies, MPSs, info) with each chain's final energy, MPS and per-sweep energies."""
    o = _resolve(options, kw)
    K = len(mpos)
    if len(chis) != K:
        raise ValueError("one bond dimension per chain")
    if o.precision not in ("f64", "ff", "mixed", "mixed-ff"):
        raise ValueError("the batched solve runs precision 'f64', 'ff', 'mixed' or 'mixed-ff'")
    if o.sites != 2 or (o.expand not in (None, 0)) or o.trunc != "svd":
        raise NotImplementedError("batched DMRG is two-site, expand=0, trunc='svd'")
    charges = list(charges) if charges is not None else [None] * K
    seeds = list(seeds) if seeds is not None else [o.seed] * K
    device = torch.device(o.device) if o.device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    import dataclasses
    chains = []
    for c in range(K):
        oc = dataclasses.replace(o, charge=charges[c], seed=int(seeds[c]), init_mps=None)
        W, M, L, R, _ = setup_chain(mpos[c], int(chis[c]), oc, device)
        N = len(W)
        sweep = [(i, True) for i in range(N - 1)] + [(i, False) for i in range(N - 2, -1, -1)]
        chains.append({"W": W, "M": M, "L": L, "R": R, "N": N, "chi": int(chis[c]),
                       "sched": sweep * o.n_sweeps, "per_sweep": len(sweep), "energies": [],
                       "disc": 0.0})
    rounds = max(len(ch["sched"]) for ch in chains)
    phase = {"eig": 0.0, "trunc": 0.0, "env": 0.0}
    stats = {"matvecs": 0, "matvecs_lo": 0}
    E_last = np.full(K, np.nan)
    main = torch.cuda.current_stream(device)

    def eig(act, r):
        """Round r's local problems of the chains `act`, solved together (main thread, main
        stream). Returns what the truncation needs."""
        t0 = time.perf_counter()
        probs, thetas = [], []
        for c in act:
            ch = chains[c]
            i, _ = ch["sched"][r]
            th = ops.tensordot(ch["M"][i], ch["M"][i + 1], 1)
            thetas.append(th)
            probs.append((th.layout, ch["L"][i], ch["W"][i], ch["W"][i + 1], ch["R"][i + 2]))
        x0 = torch.cat([t.data for t in thetas])
        mi = o.max_iter if o.max_iter is not None else max(
            min(t.layout.size, max(200, 4 * chains[c]["chi"])) for c, t in zip(act, thetas))
        hi = "ff" if o.precision in ("ff", "mixed-ff") else "f64"
        if o.precision in ("mixed", "mixed-ff"):
            # every chain's problem on the tensor cores first (split TF32, the batched plan's
            # tcgen05 operator) to tol_lo, then polished at `hi` from those vectors
            op_lo = BatchedTwoSiteOperator(probs, precision="tc")
            _, x0, info_lo = lanczos_ground_batched(op_lo, x0, op_lo.offsets,
                                                    tol=o.mixed_tol_lo, max_iter=mi,
                                                    m=o.restart_m, k=o.restart_k)
            op_lo.tc.check_device_error()
            stats["matvecs_lo"] += info_lo["matvecs"]
        op = BatchedTwoSiteOperator(probs, precision=hi)
        E, X, info = lanczos_ground_batched(op, x0, op.offsets, tol=o.eig_tol, max_iter=mi,
                                            m=o.restart_m, k=o.restart_k)
        stats["matvecs"] += info["matvecs"]
        phase["eig"] += time.perf_counter() - t0
        return act, r, E, X, op.offsets.copy(), [t.layout for t in thetas]

    def trunc_env(act, r, E, X, offsets, layouts):
        """Truncation and environment update of the chains `act` after round r, on the calling
        thread's current stream."""
        t0 = time.perf_counter()
        fused = [LA.fuse_matrix(BlockTensor(lay, X[int(a):int(b)]), 2)
                 for lay, a, b in zip(layouts, offsets[:-1], offsets[1:])]
        facs = LA.truncated_svd_many(
            [(mat, chains[c]["chi"], "right" if chains[c]["sched"][r][1] else "left")
             for (mat, _), c in zip(fused, act)], driver=o.svd_driver, method=o.svd_method,
            host=o.svd_host)
        new = []
        for (U, S, Vh, disc), (_, finfo), c in zip(facs, fused, act):
            ch = chains[c]
            i, _ = ch["sched"][r]
            ch["M"][i] = LA.split_rows(U, finfo)
            ch["M"][i + 1] = LA.split_cols(Vh, finfo)
            ch["disc"] += disc
            new += [ch["M"][i], ch["M"][i + 1]]
        torch.cuda.current_stream().synchronize()
        t1 = time.perf_counter()
        phase["trunc"] += t1 - t0
        for q, c in enumerate(act):
            ch = chains[c]
            i, right = ch["sched"][r]
            if right:
                ch["L"][i + 1] = ops.update_left_env(ch["L"][i], ch["M"][i], ch["W"][i])
                new.append(ch["L"][i + 1])
            else:
                ch["R"][i + 1] = ops.update_right_env(ch["R"][i + 2], ch["M"][i + 1],
                                                      ch["W"][i + 1])
                new.append(ch["R"][i + 1])
            E_last[c] = E[q]
            if (r + 1) % ch["per_sweep"] == 0:
                ch["energies"].append(float(E[q]))
        torch.cuda.current_stream().synchronize()
        phase["env"] += time.perf_counter() - t1
        return new

    t_wall = time.perf_counter()
    if not pipeline:
        for r in range(rounds):
            act = [c for c in range(K) if r < len(chains[c]["sched"])]
            res = eig(act, r)
            main.synchronize()
            trunc_env(*res)
    else:
        # two groups of chains, balanced by their local problems' size; while one group's
        # Lanczos runs on the main stream, the other's truncation and environment updates run
        # on a worker thread and its own stream (host LAPACK and cuSOLVER waits overlap the
        # GPU matvecs); CUDA events order each chain's rounds across the two streams
        import concurrent.futures as cf
        size = [ch["N"] * ch["chi"] ** 2 * len(ch["sched"]) for ch in chains]
        order = sorted(range(K), key=lambda c: -size[c])
        groups = [order[0::2], order[1::2]]
        side = torch.cuda.Stream(device)
        pool = cf.ThreadPoolExecutor(1, thread_name_prefix="tnk-batch")
        pending = [None, None]

        def side_task(res, ev):
            with torch.cuda.stream(side):
                side.wait_event(ev)
                res[3].record_stream(side)
                new = trunc_env(*res)
                for t in new:
                    t.data.record_stream(main)
                done = torch.cuda.Event()
                done.record(side)
                return done
        try:
            for r in range(rounds):
                for g in (0, 1):
                    act = [c for c in groups[g] if r < len(chains[c]["sched"])]
                    if pending[g] is not None:
                        main.wait_event(pending[g].result())
                        pending[g] = None
                    if not act:
                        continue
                    res = eig(act, r)
                    ev = torch.cuda.Event()
                    ev.record(main)
                    pending[g] = pool.submit(side_task, res, ev)
            for g in (0, 1):
                if pending[g] is not None:
                    main.wait_event(pending[g].result())
        finally:
            pool.shutdown(wait=True)
        main.synchronize()
    energies = [float(e) for e in E_last]
    return energies, [ch["M"] for ch in chains], {
        "energies": [ch["energies"] for ch in chains], "rounds": rounds,
        "matvecs": stats["matvecs"], "matvecs_lo": stats["matvecs_lo"], "phase_time": phase,
        "wall_s": time.perf_counter() - t_wall, "pipeline": pipeline,
        "discarded_weight": [ch["disc"] for ch in chains]}
