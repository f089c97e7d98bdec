"""Block linear algebra on the GPU around the hot path: fuse/split of legs, the block truncated
SVD with the global cut across sectors, the per-block LQ of the initial canonicalisation, norms.

  fuse_matrix / split_*   tnkit/blocks.py:1196-1286 (consecutive leg groups), as one
                          tnk_combine_f64 launch each (one unit term per block piece)
  truncated_svd           tnkit/blocks.py:1380-1462 (svd_tol = 0, degenerate_tol = 0): per-sector
                          SVD, the chi largest values over all sectors in the stable order of
                          (-sigma, position), new bond sectors labelled by the row charge
  lq                      tnkit/blocks.py:1465-1495 (right=True)

Factorisations. method='gram' on FP64 CUDA blocks cut the way a sweep cuts (scale 'right' /
'left') takes the device route (_gram_device_many): every sector's Gram matrix, Householder
reduction to tridiagonal form, back-transformation of the kept vectors and other factor on the
GPU in a handful of launches for the whole bond (csrc/sytrd.cu, grouped GEMMs), the tridiagonal
eigenproblems on host threads (hostlapack.py, O(n^2) each), the cut on the host. Otherwise the
Gram route is one library call per sector (tnk_svd_gram_f64 on cuSOLVER, from a thread pool
with one stream per sector, optionally with a host LAPACK share); 'svd' and complex blocks go
through torch.linalg. Only the singular values (and, on the device route, the tridiagonals and
the kept tridiagonal eigenvectors) cross between host and device, once per bond.
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes as C
import os
import threading
from typing import Tuple

import numpy as np
import torch

from . import _lib
from . import plan as P
from .layout import Layout, Leg, canonical
from .ops import DeviceCombPlan, _PLANS
from .tensor import BlockTensor


def _fuse_info(layout: Layout, nrow: int) -> P.FuseInfo:
    return _PLANS.get_or(("fuseinfo", layout, nrow), lambda: P.FuseInfo(layout, nrow))


def _comb_plan(key, build, data):
    """Device combination plan for `data`'s dtype (complex128: re/im halves separately)."""
    cplx = data.is_complex()

    def make():
        hp = build()
        if cplx:
            c = P.HostCombPlan.__new__(P.HostCombPlan)
            c.c, c.out_layout, c.extra = P.complexify_comb(hp.c), hp.out_layout, hp.extra
            hp = c
        return DeviceCombPlan(hp, data.device)
    return _PLANS.get_or(key + (str(data.device), cplx), make)


def fuse_matrix(t: BlockTensor, nrow: int) -> Tuple[BlockTensor, P.FuseInfo]:
    """Fuse legs [0, nrow) and [nrow, n) of `t` into a two-leg block matrix."""
    info = _fuse_info(t.layout, nrow)
    p = _comb_plan(("fuse", t.layout, nrow), lambda: P.plan_fuse(info), t.data)
    out = torch.empty(info.matrix.size, dtype=t.data.dtype, device=t.data.device)
    p.run(t.data, out)
    return BlockTensor(info.matrix, out), info


def split_rows(m: BlockTensor, info: P.FuseInfo) -> BlockTensor:
    p = _comb_plan(("split_r", info.layout, info.nrow, m.layout),
                   lambda: P.plan_split_rows(info, m.layout), m.data)
    out = torch.empty(p.out_layout.size, dtype=m.data.dtype, device=m.data.device)
    p.run(m.data, out)
    return BlockTensor(p.out_layout, out)


def split_cols(m: BlockTensor, info: P.FuseInfo) -> BlockTensor:
    p = _comb_plan(("split_c", info.layout, info.nrow, m.layout),
                   lambda: P.plan_split_cols(info, m.layout), m.data)
    out = torch.empty(p.out_layout.size, dtype=m.data.dtype, device=m.data.device)
    p.run(m.data, out)
    return BlockTensor(p.out_layout, out)


def _blocks(m: BlockTensor):
    lay = m.layout
    for k in range(lay.nblocks):
        r, c = lay.key(k)
        R, Cc = lay.shape(k)
        o = int(lay.offsets[k])
        yield r, c, m.data[o:o + R * Cc].view(R, Cc)


def _row_label(leg: Leg, r: int):
    q = leg.charges[r]
    if leg.sign > 0:
        return q
    return tuple(-x for x in q) if isinstance(q, tuple) else -q


class _Concurrent:
    """Per-sector factorisations issued from a thread pool, one CUDA stream per sector: the
    cuSOLVER calls of one bond (a dozen sectors of a few hundred rows at chi = 1024) are
    latency-bound one by one and overlap well."""

    def __init__(self, workers: int = 16):
        self.pool = cf.ThreadPoolExecutor(workers, thread_name_prefix="tnk-svd")
        self.streams = {}
        self.lock = threading.Lock()
        self.warmed = set()

    def stream(self, device, i):
        with self.lock:
            key = (str(device), i)
            if key not in self.streams:
                self.streams[key] = torch.cuda.Stream(device=device)
            return self.streams[key]

    def _warm(self, device):
        """torch.linalg's CUDA libraries are loaded lazily, and the first call must not come
        from several threads at once (torch raises "lazy wrapper should be called at most
        once"): make the first calls here, on the calling thread, once per device."""
        key = str(device)
        if key in self.warmed:
            return
        a = torch.eye(2, dtype=torch.float64, device=device)
        torch.linalg.qr(a)
        torch.linalg.eigh(a)
        torch.linalg.svd(a, full_matrices=False)
        self.warmed.add(key)

    def map(self, fn, mats, device):
        """fn(M) for each M (or fn[i](M_i) when fn is a list), one stream per item."""
        self._warm(device)
        main = torch.cuda.current_stream(device)
        streams = [self.stream(device, i) for i in range(len(mats))]
        for s in streams:
            s.wait_stream(main)
        fns = fn if isinstance(fn, (list, tuple)) else [fn] * len(mats)

        def keep(out):
            for t in out:
                if isinstance(t, torch.Tensor):
                    t.record_stream(main)
                elif isinstance(t, (list, tuple)):
                    keep(t)

        def run(i):
            with torch.cuda.stream(streams[i]):
                out = fns[i](mats[i])
                keep(out)
                return out
        res = list(self.pool.map(run, range(len(mats))))
        for s in streams:
            main.wait_stream(s)
        return res


_CONC = None


def _concurrent() -> _Concurrent:
    global _CONC
    if _CONC is None:
        _CONC = _Concurrent()
    return _CONC


def _svd_gram_native(M: torch.Tensor, orth: int = 0):
    """U, S, Vh (and S on the host) of one real CUDA block (FP64, or FP32) by
    tnk_svd_gram_f64 / _f32: the same factorisation as _svd_gram in one library call that holds
    no interpreter lock. orth = 1 / 2 (FP64): the U / Vh side straight from its own Gram matrix,
    no QR (tnk_svd_gram2_f64)."""
    R, Cc = M.shape
    k = min(R, Cc)
    lib = _lib.lib()
    f32 = M.dtype == torch.float32
    nb = C.c_int64()
    if orth and not f32:
        _lib.check(lib.tnk_svd_gram_ws2_f64(R, Cc, orth, C.byref(nb)), "svd_gram_ws")
        call = lambda *a: lib.tnk_svd_gram2_f64(a[0], R, Cc, orth, *a[1:])
    else:
        ws_fn, fn = ((lib.tnk_svd_gram_ws_f32, lib.tnk_svd_gram_f32) if f32 else
                     (lib.tnk_svd_gram_ws_f64, lib.tnk_svd_gram_f64))
        _lib.check(ws_fn(R, Cc, C.byref(nb)), "svd_gram_ws")
        call = lambda *a: fn(a[0], R, Cc, *a[1:])
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=M.device)
    U = torch.empty((R, k), dtype=M.dtype, device=M.device)
    S = torch.empty(k, dtype=M.dtype, device=M.device)
    Vh = torch.empty((k, Cc), dtype=M.dtype, device=M.device)
    s_host = np.empty(k, dtype=np.float64)
    _lib.check(call(M.data_ptr(), U.data_ptr(), S.data_ptr(), Vh.data_ptr(), ws.data_ptr(),
                    ws.numel(), s_host.ctypes.data, _lib.stream_ptr()), "svd_gram")
    return U, S, Vh, s_host


# --- host co-processing of the per-sector route ------------------------------------------------
# (host='auto' where the device route does not apply, and host='always')
# A chi=1024 bond's largest sectors (~520 rows) are latency-bound in cuSOLVER: one Gram
# factorisation takes ~17 ms, and calls on several streams do not overlap (the GPU path is one
# lane). The host's cores are idle during the truncation, and host LAPACK calls from several
# threads do run side by side when each uses a share of the cores. So sectors are scheduled over
# one GPU lane and _HOST_LANES host lanes (numpy, the reference's own numpy branch of
# method='gram'; numpy releases the interpreter lock inside LAPACK), longest first, each to the
# lane that finishes it first, on costs measured on GB300 and its Grace host (522 rows: 17.3 ms
# on the GPU path, 14.0 ms on the host path with 4 of the 16 cores). Each host lane runs its
# sectors one after another with cores / _HOST_LANES library threads.
_GPU_MS_PER_ROW = 17.3 / 522          # cuSOLVER Gram path: ~linear in n (latency-bound)
_HOST_MS_522 = 14.0                   # host Gram path with cores / _HOST_LANES threads: ~n^2.1
_HOST_LANES = 4                       # host sectors in flight at once
_HOST_THREADS_DIV = _HOST_LANES       # host library threads per lane: cores / this
_HOST_BLAS = {"lib": None, "tried": False}


def _host_blas():
    """(set, get) of numpy's bundled OpenBLAS thread count, or None when not found."""
    if not _HOST_BLAS["tried"]:
        _HOST_BLAS["tried"] = True
        import glob
        import os
        base = os.path.join(os.path.dirname(os.path.dirname(np.__file__)), "numpy.libs")
        for path in sorted(glob.glob(os.path.join(base, "libscipy_openblas*.so*"))):
            try:
                lib = C.CDLL(path)
                set_, get_ = (lib.scipy_openblas_set_num_threads64_,
                              lib.scipy_openblas_get_num_threads64_)
            except (OSError, AttributeError):
                continue
            set_.argtypes, set_.restype = [C.c_int], None
            get_.argtypes, get_.restype = [], C.c_int
            _HOST_BLAS["lib"] = (set_, get_)
            break
    return _HOST_BLAS["lib"]


def _map_hybrid(fns, mats, lanes, device):
    """fns[i](mats[i]) for every sector: each GPU sector (lane -1) on its own stream and worker,
    each host lane's sectors one after another, largest first, in one worker per lane."""
    gpu = [i for i, l in enumerate(lanes) if l < 0]
    order = sorted(range(len(mats)), key=lambda i: -min(mats[i].shape))
    host = [[i for i in order if lanes[i] == k] for k in range(max(lanes, default=-1) + 1)]
    host = [ix for ix in host if ix]
    items = [fns[i] for i in gpu] + [lambda _, ix=ix: [fns[i](mats[i]) for i in ix]
                                     for ix in host]
    res = _concurrent().map(items, [mats[i] for i in gpu] + [None] * len(host), device)
    out = [None] * len(mats)
    for i, r in zip(gpu, res[:len(gpu)]):
        out[i] = r
    for ix, rs in zip(host, res[len(gpu):]):
        for i, r in zip(ix, rs):
            out[i] = r
    return out


def _assign_sectors(shapes, host_ok: bool, gpu_ok: bool = True):
    """Per sector its lane: -1 for the GPU path, 0.._HOST_LANES-1 for a host lane. Longest
    processing time first: sectors by decreasing size, each to the lane that finishes it
    first (the GPU lane alone when the host path is unavailable, host lanes alone when
    gpu_ok is False)."""
    if not host_ok or (gpu_ok and len(shapes) < 2):
        return [-1] * len(shapes)
    order = sorted(range(len(shapes)), key=lambda i: -min(shapes[i]))
    t_gpu, t_host = 0.0, [0.0] * _HOST_LANES
    out = [-1] * len(shapes)
    for i in order:
        n = min(shapes[i])
        g = _GPU_MS_PER_ROW * n + 0.4
        h = _HOST_MS_522 * (n / 522.0) ** 2.1 + 0.05
        k = min(range(_HOST_LANES), key=lambda j: t_host[j])
        if not gpu_ok or t_host[k] + h < t_gpu + g:
            out[i] = k
            t_host[k] += h
        else:
            t_gpu += g
    return out


def _svd_gram_host(M: torch.Tensor, orth: int = 0):
    """The Gram factorisation of one block on the host (numpy / LAPACK), results back on the
    device: the reference's numpy branch (tnkit/blocks.py:1345-1377), or with orth = 1 / 2 the
    canonical side straight from its own Gram matrix (as _svd_gram_native)."""
    Mh = M.cpu().numpy()
    R, Cc = Mh.shape
    dev = M.device
    if orth:
        k = min(R, Cc)
        lam, E = np.linalg.eigh(Mh @ Mh.T if orth == 1 else Mh.T @ Mh)
        lam, E = lam[::-1][:k], E[:, ::-1][:, :k]
        S = np.sqrt(np.maximum(lam, 0.0))
        inv = np.where(S > 0, 1.0 / np.where(S > 0, S, 1.0), 0.0)
        if orth == 1:
            U, Vh = E, (E.T @ Mh) * inv[:, None]
        else:
            U, Vh = (Mh @ E) * inv[None, :], E.T
        # explicit copies: a (n, 1) view with a negative stride counts as contiguous
        return (torch.as_tensor(U.copy(order="C"), device=dev),
                torch.as_tensor(S.copy(), device=dev),
                torch.as_tensor(Vh.copy(order="C"), device=dev), S.astype(np.float64))
    if R >= Cc:
        _, V = np.linalg.eigh(Mh.T @ Mh)
        V = V[:, ::-1]
        Q, Rr = np.linalg.qr(Mh @ V)
    else:
        _, Uh = np.linalg.eigh(Mh @ Mh.T)
        Uh = Uh[:, ::-1]
        Q, Rr = np.linalg.qr(Mh.T @ Uh)
    d = np.diagonal(Rr)
    S = np.abs(d)
    Q = Q * np.where(S > 0, d / np.where(S > 0, S, 1.0), 1.0)
    o = np.argsort(-S, kind="stable")
    S, Q = S[o], Q[:, o]
    if R >= Cc:
        U, Vh = Q, V[:, o].T
    else:
        U, Vh = Uh[:, o], Q.T
    return (torch.as_tensor(U.copy(order="C"), device=dev),
            torch.as_tensor(S.copy(), device=dev),
            torch.as_tensor(Vh.copy(order="C"), device=dev), S.astype(np.float64))


def _with_fp64_fallback(fn):
    """fn on an FP32 block, refactored in FP64 (results cast back) when the FP32 eigensolver
    does not converge: a Gram spectrum spanning ~18 decades can defeat it."""
    def run(M):
        try:
            return fn(M)
        except (_lib.TnkError, np.linalg.LinAlgError):
            U, S, Vh, h = fn(M.double())
            return U.float(), S.float(), Vh.float(), h
    return run


def _svd_gram(M: torch.Tensor):
    """U, S (descending), Vh of one block through the smaller Gram matrix: Hermitian eigh, then
    a QR that re-orthonormalises the computed singular vectors (the reference's method='gram',
    tnkit/blocks.py:1345-1377). Singular values below ~1e-8 of the largest are not resolved."""
    R, C = M.shape
    if R >= C:
        w, V = torch.linalg.eigh(M.mH @ M)
        V = torch.flip(V, (-1,))
        Q, Rr = torch.linalg.qr(M @ V)
    else:
        w, U = torch.linalg.eigh(M @ M.mH)
        U = torch.flip(U, (-1,))
        Q, Rr = torch.linalg.qr(M.mH @ U)
    d = torch.diagonal(Rr)
    S = d.abs()
    Q = Q * torch.where(S > 0, d / torch.where(S > 0, S, torch.ones_like(S)),
                        torch.ones_like(S))
    o = torch.argsort(S, descending=True, stable=True)
    S, Q = S[o], Q[:, o]
    if R >= C:
        return Q.contiguous(), S, V[:, o].mH.contiguous()
    return U[:, o].contiguous(), S, Q.mH.contiguous()


# --- the device Gram route --------------------------------------------------------------------
# Every sector of a bond (of several bonds: truncated_svd_many) through its canonical side's Gram
# matrix, G = M M^T for scale 'right' (U from its eigenvectors), M^T M for 'left' (Vh from its
# eigenvectors), the smaller one for 'none': the Gram matrices by cuBLAS, their reduction to
# tridiagonal form in one launch (tnk_sytrd_batched_f64), the tridiagonal eigenproblems on the
# host (hostlapack.tridiag_eigh_many, O(n^2) each), the global cut, then the back-transformation
# of only the kept eigenvectors in one launch (tnk_ormtr_batched_f64) and the other factor as the
# exact projection, diag(1/S) U^T M or M V diag(1/S). Sectors larger than the reduction takes
# go through _svd_gram_native.
_SYTRD = {"limits": None}
# time model of one sector's reduction with a cluster of cs CTAs: ~n^3 FP64 FMAs shared by the
# cluster, plus a fixed cost per column (two cluster barriers and the gathers; one CTA barrier
# pair when cs = 1), measured on GB300
_SY_FMA_PER_S = 3.6e9                 # FP64 FMAs per second per SM
_SY_STEP_S = {1: 0.6e-6, 2: 1.4e-6, 4: 1.5e-6, 8: 1.6e-6, 16: 1.8e-6}


def _sytrd_table():
    """{cluster size: largest order} of the device reduction on the current device (0: that
    cluster size cannot launch there)."""
    if _SYTRD["limits"] is None:
        lib = _lib.lib()
        lim = {}
        for cs in (1, 2, 4, 8, 16):
            nm = C.c_int32(0)
            _lib.check(lib.tnk_sytrd_limits(cs, C.byref(nm)), "tnk_sytrd_limits")
            lim[cs] = int(nm.value)
        _SYTRD["limits"] = lim
    return _SYTRD["limits"]


def _sytrd_limits():
    """(largest usable cluster size, its largest order) of the device reduction."""
    lim = _sytrd_table()
    for cs in (16, 8, 4, 2, 1):
        if lim[cs] > 0:
            return cs, lim[cs]
    return 0, 0


def _sy_time(n: int, cs: int) -> float:
    return n ** 3 / (cs * _SY_FMA_PER_S) + n * _SY_STEP_S[cs]


def _sytrd_clusters(ns, n_sm: int):
    """A cluster size per sector order: each sector's fastest alone, then, while the clusters
    need more than one wave of the SMs, the sector whose halving costs least in makespan terms
    gets half the CTAs (throughput for many small sectors, latency for a bond's few large
    ones)."""
    lim = _sytrd_table()
    ok = lambda n, c: lim.get(c, 0) >= n
    cs = []
    for n in ns:
        cands = [c for c in (1, 2, 4, 8, 16) if ok(n, c)]
        cs.append(min(cands, key=lambda c: _sy_time(n, c)) if cands else 0)
    while sum(cs) > n_sm:
        best, cost = None, None
        for i, (n, c) in enumerate(zip(ns, cs)):
            if c > 1 and ok(n, c // 2):
                d = _sy_time(n, c // 2) - _sy_time(n, c)
                if cost is None or d < cost:
                    best, cost = i, d
        if best is None:
            break
        cs[best] //= 2
    return cs


def device_gram_available() -> bool:
    """Whether the device Gram route can run here (a CUDA device with the cluster launch, and
    the host tridiagonal solver)."""
    from . import hostlapack
    if not torch.cuda.is_available() or not hostlapack.available():
        return False
    return _sytrd_limits()[1] > 0


# host threads for the tridiagonal eigenproblems of one pass (each O(n^2) with deflation)
_STEDC_LANES = max(1, min(8, (os.cpu_count() or 2) // 2))


def _gram_side(scale: str, R: int, Cc: int) -> int:
    return 1 if scale == "right" else 2 if scale == "left" else (1 if R <= Cc else 2)


_PIN = {"buf": None, "done": None}


def _pinned(nelem: int) -> torch.Tensor:
    """A page-locked FP64 host buffer of at least nelem entries, reused across calls (the copy
    that last read it has finished when it is handed out again)."""
    if _PIN["done"] is not None:
        _PIN["done"].synchronize()
    buf = _PIN["buf"]
    if buf is None or buf.numel() < nelem:
        buf = torch.empty(max(nelem, 2 * (buf.numel() if buf is not None else 0), 1 << 16),
                          dtype=torch.float64, pin_memory=True)
        _PIN["buf"] = buf
    return buf


def _product_tables(prods, upper_only=False):
    """Task, segment and tile tables (numpy, the tnk_gemm_* layouts) of several products
    C_p = A_p B_p with C row-major (C(i, j) at c_off + i ldc + j): prods holds per product
    (c_off, ldc, m, n, k, (a_buf, a_off, a_rs, a_cs), (b_buf, b_off, b_rs, b_cs)). With
    upper_only, only the tiles that hold entries with i <= j (square symmetric outputs of which
    only that triangle is read -- the lower triangle of the column-major view). Tiles longest K
    first."""
    from ._lib import GEMM_SEG, GEMM_TASK, GEMM_TILE
    from .plan import TILE_M, TILE_N
    tasks = np.zeros(len(prods), dtype=GEMM_TASK)
    segs = np.zeros(len(prods), dtype=GEMM_SEG)
    tiles = []
    for t, (c_off, ldc, m, n, k, a, b) in enumerate(prods):
        tasks[t] = (c_off, ldc, m, n, t, t + 1, 0)
        segs[t] = (a[1], b[1], a[2], a[3], b[2], b[3], k, a[0], b[0], 0, 0, 1.0)
        for m0 in range(0, m, TILE_M):
            for n0 in range(0, n, TILE_N):
                if upper_only and m0 > n0 + TILE_N - 1:
                    continue
                tiles.append((k, t, m0, n0))
    tiles.sort(key=lambda x: -x[0])
    tl = np.zeros(len(tiles), dtype=GEMM_TILE)
    if tiles:
        arr = np.asarray(tiles, dtype=np.int64)
        tl["task"], tl["m0"], tl["n0"] = arr[:, 1], arr[:, 2], arr[:, 3]
    return tasks, segs, tl


def _grouped_products(prods, C_out: torch.Tensor, slots, upper_only=False):
    """One tnk_grouped_gemm_f64 launch of _product_tables(prods, upper_only) with operand slots
    `slots` (device addresses) and output base C_out. Returns the table tensor (to be kept
    alive until the stream has run the launch)."""
    tasks, segs, tl = _product_tables(prods, upper_only)
    host = np.concatenate([tasks.view(np.uint8), segs.view(np.uint8), tl.view(np.uint8)])
    dt = torch.from_numpy(host).to(C_out.device)
    a0, a1 = tasks.nbytes, tasks.nbytes + segs.nbytes
    sl = list(slots) + [0] * (4 - len(slots))
    _lib.check(_lib.lib().tnk_grouped_gemm_f64(dt.data_ptr(), dt.data_ptr() + a0,
                                               dt.data_ptr() + a1, len(tl), sl[0], sl[1], sl[2],
                                               sl[3], C_out.data_ptr(), _lib.stream_ptr()),
               "tnk_grouped_gemm_f64")
    return dt


def _gram_products(sectors):
    """The Gram products of the device route for [(offset of M in slot 0, R, C, side,
    offset of G)]: G = M M^T (side 1) or M^T M (side 2), n x n."""
    prods = []
    for mo, R, Cc, side, go in sectors:
        n = R if side == 1 else Cc
        if side == 1:          # A = M (R x C), B(k, j) = M[j, k]
            prods.append((go, n, n, n, Cc, (0, mo, Cc, 1), (0, mo, 1, Cc)))
        else:                  # A(i, k) = M[k, i], B = M
            prods.append((go, n, n, n, R, (0, mo, 1, Cc), (0, mo, Cc, 1)))
    return prods


def _other_products(sectors):
    """The other factor's products for [(offset of M in slot 0, R, C, side, offset of V in
    slot 1, q kept, offset of the output)]: side 1: V (q x R) M, q x C; side 2: M V^T
    (V q x C), R x q."""
    prods = []
    for mo, R, Cc, side, zo, q, po in sectors:
        if side == 1:
            prods.append((po, Cc, q, Cc, R, (1, zo, R, 1), (0, mo, Cc, 1)))
        else:
            prods.append((po, q, R, q, Cc, (0, mo, Cc, 1), (1, zo, 1, Cc)))
    return prods


def _gram_device_many(items, timing=None):
    """[(m, blocks, chi, scale, normalize)] -> [(U, S, Vh, disc)] by the device Gram route.
    With a dict `timing`, the phases' times in ms are added to it (CUDA events for the device
    phases, host clock for the host one; the call then synchronises at its end)."""
    import time
    from . import hostlapack
    lib = _lib.lib()
    ev = {}

    def mark(name):
        if timing is not None:
            ev[name] = torch.cuda.Event(enable_timing=True)
            ev[name].record()
    cs_max, nmax = _sytrd_limits()
    if nmax <= 0:
        raise RuntimeError("the device Gram route needs thread-block clusters on a CUDA device")
    dev = items[0][0].data.device
    sp = _lib.stream_ptr()
    keep = []                   # tables and buffers the stream still reads
    sec = []                    # (item, block index, M, side, n)
    for it, (m, blocks, chi, scale, normalize) in enumerate(items):
        for b, (_, _, M) in enumerate(blocks):
            R, Cc = M.shape
            side = _gram_side(scale, R, Cc)
            sec.append((it, b, M, side, R if side == 1 else Cc))
    on_dev = sorted([i for i, s in enumerate(sec) if s[4] <= nmax], key=lambda i: -sec[i][4])
    off_dev = [i for i, s in enumerate(sec) if s[4] > nmax]
    base = min(s[2].data_ptr() for s in sec)          # operand slot 0: the blocks' buffers
    moff = {i: (s[2].data_ptr() - base) // 8 for i, s in enumerate(sec)}
    # Gram matrices, packed; the reduction reads the lower triangle of the column-major view,
    # which is the upper one of the row-major products written here
    tab = np.zeros((max(len(on_dev), 1), 4), dtype=np.int64)
    g = v = 0
    for r, i in enumerate(on_dev):
        n = sec[i][4]
        tab[r, :3] = (n, g, v)
        g += n * n
        v += n
    G = torch.empty(max(g, 1), dtype=torch.float64, device=dev)
    dv = torch.empty(3 * max(v, 1), dtype=torch.float64, device=dev)
    d, e, tau = dv[:max(v, 1)], dv[max(v, 1):2 * max(v, 1)], dv[2 * max(v, 1):]
    mark("gram0")
    prods = _gram_products([(moff[i], sec[i][2].shape[0], sec[i][2].shape[1], sec[i][3],
                             int(tab[r, 1])) for r, i in enumerate(on_dev)])
    if prods:
        keep.append(_grouped_products(prods, G, [base], upper_only=True))
    facs = {}
    if on_dev:
        # one launch per cluster size, each over its sectors (largest first)
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        cls = _sytrd_clusters([int(tab[r, 0]) for r in range(len(on_dev))], n_sm)
        main = torch.cuda.current_stream(dev)
        mark("red0")
        for j, c in enumerate(sorted(set(cls), reverse=True)):
            rows = [r for r in range(len(on_dev)) if cls[r] == c]
            sub = torch.from_numpy(np.ascontiguousarray(tab[rows])).to(dev)
            st = main if j == 0 else _concurrent().stream(dev, 64 + j)
            if st is not main:
                st.wait_stream(main)
            with torch.cuda.stream(st):
                _lib.check(lib.tnk_sytrd_batched_f64(
                    sub.data_ptr(), len(rows), int(tab[rows, 0].max()), c, G.data_ptr(),
                    d.data_ptr(), e.data_ptr(), tau.data_ptr(), _lib.stream_ptr()),
                    "tnk_sytrd_batched_f64")
                sub.record_stream(st)
            if st is not main:
                main.wait_stream(st)
        mark("red1")
        t_host = time.perf_counter()
        de = dv[:2 * max(v, 1)].cpu().numpy()
        dh, eh = de[:max(v, 1)], de[max(v, 1):]
    # sectors too large for the reduction, meanwhile on the GPU path
    for i in off_dev:
        _, _, M, side, _ = sec[i]
        facs[i] = _svd_gram_native(M, side)
    if on_dev:
        eig = hostlapack.tridiag_eigh_many(
            [(dh[tab[r, 2]:tab[r, 2] + tab[r, 0]], eh[tab[r, 2]:tab[r, 2] + tab[r, 0]])
             for r in range(len(on_dev))], lanes=_STEDC_LANES)
    sig = {}
    for r, i in enumerate(on_dev):
        M = sec[i][2]
        k = min(M.shape)
        lam = eig[r][0][::-1][:k]
        sig[i] = np.sqrt(np.maximum(lam, 0.0))
    for i in off_dev:
        sig[i] = facs[i][3]
    # the cut of each item (the rule of _trunc_finish), then the kept eigenvectors to the device
    kept = {}
    for it, (m, blocks, chi, scale, normalize) in enumerate(items):
        ids = [i for i, s in enumerate(sec) if s[0] == it]
        cnt = _cut([sig[i] for i in ids], chi)[0]
        for j, i in enumerate(ids):
            kept[i] = int(cnt[j])
    # back-transformation items: column chunks of up to 8 (one warp each); a bond whose kept
    # columns would not give every SM two CTAs gets chunks of 2, so its largest sectors spread
    # over more SMs (the work is FP64-bound, ~n^2 FMAs per column)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    chunk = 8 if sum((kept[i] + 7) // 8 for i in on_dev) >= 2 * n_sm else 2
    z = ns = 0
    items_orm = []
    for r, i in enumerate(on_dev):
        n, q = int(tab[r, 0]), kept[i]
        tab[r, 3] = z
        if q:
            for c0 in range(0, q, chunk):
                items_orm.append((r, c0, min(chunk, q - c0), 0))
            z += q * n
            ns += q
    if z:
        # kept eigenvectors (descending) and their S through one page-locked buffer
        pin = _pinned(z + ns)
        hz = pin.numpy()
        so = z
        for r, i in enumerate(on_dev):
            n, q = int(tab[r, 0]), kept[i]
            if q:
                Zf = eig[r][1]
                o = int(tab[r, 3])
                hz[o:o + q * n].reshape(q, n)[:] = Zf[:, n - q:][:, ::-1].T
                hz[so:so + q] = sig[i][:q]
                so += q
        up = torch.empty(z + ns, dtype=torch.float64, device=dev)
        up.copy_(pin[:z + ns], non_blocking=True)
        _PIN["done"] = torch.cuda.Event()
        _PIN["done"].record()
        if timing is not None:
            timing["host_ms"] = timing.get("host_ms", 0.0) + (time.perf_counter() - t_host) * 1e3
        Zd, S_all = up[:z], up[z:]
        tab_z = torch.from_numpy(tab).to(dev)
        it_d = torch.from_numpy(np.asarray(items_orm, dtype=np.int32)).to(dev)
        keep += [tab_z, it_d]
        mark("back0")
        _lib.check(lib.tnk_ormtr_batched_f64(tab_z.data_ptr(), it_d.data_ptr(), len(items_orm),
                                             int(tab[:, 0].max()), G.data_ptr(), tau.data_ptr(),
                                             Zd.data_ptr(), sp), "tnk_ormtr_batched_f64")
        mark("back1")
        inv_all = torch.where(S_all > 0, 1.0 / torch.where(S_all > 0, S_all,
                                                            torch.ones_like(S_all)),
                              torch.zeros_like(S_all))
        # the other factor of every sector in one launch: diag(1/S) V M or M V^T diag(1/S)
        osec, poff, p = [], {}, 0
        for r, i in enumerate(on_dev):
            _, _, M, side, n = sec[i]
            q = kept[i]
            if not q:
                continue
            R, Cc = M.shape
            poff[i] = p
            osec.append((moff[i], R, Cc, side, int(tab[r, 3]), q, p))
            p += q * (Cc if side == 1 else R)
        prods = _other_products(osec)
        P_all = torch.empty(max(p, 1), dtype=torch.float64, device=dev)
        keep.append(_grouped_products(prods, P_all, [base, Zd.data_ptr()]))
        mark("other1")
    elif on_dev and timing is not None:
        timing["host_ms"] = timing.get("host_ms", 0.0) + (time.perf_counter() - t_host) * 1e3
    so = 0
    for r, i in enumerate(on_dev):
        _, _, M, side, n = sec[i]
        q = kept[i]
        R, Cc = M.shape
        if not q:
            facs[i] = (M.new_zeros((R, 0)), M.new_zeros(0), M.new_zeros((0, Cc)), sig[i])
            continue
        V = Zd[int(tab[r, 3]):int(tab[r, 3]) + q * n].view(q, n)   # row j: eigenvector j of G
        S, inv = S_all[so:so + q], inv_all[so:so + q]
        so += q
        if side == 1:
            Vh = P_all[poff[i]:poff[i] + q * Cc].view(q, Cc)
            Vh.mul_(inv[:, None])
            facs[i] = (V.mT, S, Vh, sig[i])
        else:
            U = P_all[poff[i]:poff[i] + R * q].view(R, q)
            U.mul_(inv[None, :])
            facs[i] = (U, S, V, sig[i])
    out = []
    for it, (m, blocks, chi, scale, normalize) in enumerate(items):
        ids = [i for i, s in enumerate(sec) if s[0] == it]
        out.append(_trunc_finish(m, blocks, [facs[i] for i in ids], chi, scale, normalize))
    if timing is not None:
        mark("end")
        torch.cuda.synchronize(dev)
        span = lambda a, b: ev[a].elapsed_time(ev[b]) if a in ev and b in ev else 0.0
        for k, (a, b) in {"gram_ms": ("gram0", "red0"), "reduce_ms": ("red0", "red1"),
                          "back_ms": ("back0", "back1"), "other_ms": ("back1", "other1"),
                          "total_ms": ("gram0", "end")}.items():
            timing[k] = timing.get(k, 0.0) + span(a, b)
        timing["sectors"] = len(sec)
        timing["sectors_on_device"] = len(on_dev)
        timing["reduce_flops"] = timing.get("reduce_flops", 0.0) + sum(
            4.0 / 3.0 * sec[i][4] ** 3 for i in on_dev)
    return out


# --- the device exact route --------------------------------------------------------------------
# Every sector's exact SVD (the reference's default method='svd') as LAPACK's dgesdd computes
# it: the Householder bidiagonalisation of the block (or its transpose, m >= n) in one launch per
# cluster size (tnk_gebrd_batched_f64), the bidiagonal SVDs on host threads
# (hostlapack.bidiag_svd_many, O(n^2) each), the global cut, then the back-transformation of the
# kept left and right singular vectors in one launch (tnk_ormqr_batched_f64). Sectors larger
# than the reduction takes go through torch.linalg.svd.
_GEBRD = {"limits": None}
_GB_STEP_S = {1: 1.0e-6, 2: 2.6e-6, 4: 2.7e-6, 8: 2.8e-6, 16: 3.0e-6}


def _gebrd_table():
    if _GEBRD["limits"] is None:
        lib = _lib.lib()
        lim = {}
        for cs in (1, 2, 4, 8, 16):
            nm = C.c_int32(0)
            _lib.check(lib.tnk_gebrd_limits(cs, C.byref(nm)), "tnk_gebrd_limits")
            lim[cs] = int(nm.value)
        _GEBRD["limits"] = lim
    return _GEBRD["limits"]


def device_svd_available() -> bool:
    """Whether the device exact route can run here."""
    from . import hostlapack
    if not torch.cuda.is_available() or not hostlapack.available():
        return False
    return max(_gebrd_table().values()) > 0


def _gebrd_clusters(shapes, n_sm: int):
    """A cluster size per (m, n) block (m >= n), as _sytrd_clusters chooses them: each block's
    fastest alone by a time model (~4 m n^2 FP64 FMAs over the cluster, four cluster barriers
    per column), then halvings while the clusters need more than one wave of the SMs."""
    lim = _gebrd_table()
    ok = lambda m, c: lim.get(c, 0) >= m
    t = lambda m, n, c: 4.0 * (m * n * n - n ** 3 / 3.0) / (c * _SY_FMA_PER_S) + n * _GB_STEP_S[c]
    cs = []
    for m, n in shapes:
        cands = [c for c in (1, 2, 4, 8, 16) if ok(m, c)]
        cs.append(min(cands, key=lambda c: t(m, n, c)) if cands else 0)
    while sum(cs) > n_sm:
        best, cost = None, None
        for i, ((m, n), c) in enumerate(zip(shapes, cs)):
            if c > 1 and ok(m, c // 2):
                dlt = t(m, n, c // 2) - t(m, n, c)
                if cost is None or dlt < cost:
                    best, cost = i, dlt
        if best is None:
            break
        cs[best] //= 2
    return cs


def _svd_device_many(items, timing=None):
    """[(m, blocks, chi, scale, normalize)] -> [(U, S, Vh, disc)] by the device exact route
    (see above). With a dict `timing`, phase times in ms are added to it."""
    import time
    from . import hostlapack
    from ._lib import GEBRD_SECTOR, REFL_SET
    lib = _lib.lib()
    ev = {}

    def mark(name):
        if timing is not None:
            ev[name] = torch.cuda.Event(enable_timing=True)
            ev[name].record()
    lim = _gebrd_table()
    mmax_dev = max(lim.values())
    if mmax_dev <= 0:
        raise RuntimeError("the device exact route needs thread-block clusters on a CUDA device")
    dev = items[0][0].data.device
    sp = _lib.stream_ptr()
    keep = []
    sec = []                    # (item, block index, M, transposed, m, n)
    for it, (mt, blocks, chi, scale, normalize) in enumerate(items):
        for b, (_, _, M) in enumerate(blocks):
            R, Cc = M.shape
            tr = R < Cc
            sec.append((it, b, M, tr, max(R, Cc), min(R, Cc)))
    on_dev = sorted([i for i, s in enumerate(sec) if s[4] <= mmax_dev],
                    key=lambda i: -(sec[i][4] * sec[i][5] ** 2))
    off_dev = [i for i, s in enumerate(sec) if s[4] > mmax_dev]
    base = min(s[2].data_ptr() for s in sec)
    tab = np.zeros(max(len(on_dev), 1), dtype=GEBRD_SECTOR)
    refl = vo = 0
    for r, i in enumerate(on_dev):
        _, _, M, tr, mm, nn = sec[i]
        Cc = M.shape[1]
        tab[r] = (mm, nn, (M.data_ptr() - base) // 8, refl, refl + mm * nn, vo, 0,
                  1 if tr else Cc, Cc if tr else 1)
        refl += mm * nn + nn * nn
        vo += 4 * nn
    RF = torch.empty(max(refl, 1), dtype=torch.float64, device=dev)
    vec = torch.zeros(max(vo, 1), dtype=torch.float64, device=dev)
    facs = {}
    if on_dev:
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        cls = _gebrd_clusters([(int(tab[r]["m"]), int(tab[r]["n"])) for r in range(len(on_dev))],
                              n_sm)
        main = torch.cuda.current_stream(dev)
        mark("red0")
        for j, c in enumerate(sorted(set(cls), reverse=True)):
            rows = [r for r in range(len(on_dev)) if cls[r] == c]
            sub_h = np.ascontiguousarray(tab[rows])
            sub = torch.from_numpy(sub_h.view(np.uint8)).to(dev)
            st = main if j == 0 else _concurrent().stream(dev, 80 + j)
            if st is not main:
                st.wait_stream(main)
            with torch.cuda.stream(st):
                _lib.check(lib.tnk_gebrd_batched_f64(
                    sub.data_ptr(), len(rows), int(sub_h["m"].max()), int(sub_h["n"].max()), c,
                    base, RF.data_ptr(), RF.data_ptr(), vec.data_ptr(), _lib.stream_ptr()),
                    "tnk_gebrd_batched_f64")
                sub.record_stream(st)
            if st is not main:
                main.wait_stream(st)
        mark("red1")
        t_host = time.perf_counter()
        vh = vec.cpu().numpy()
    for i in off_dev:
        M = sec[i][2]
        U, S, Vh = torch.linalg.svd(M, full_matrices=False)
        facs[i] = (U, S, Vh, S.cpu().numpy().astype(np.float64))
    if on_dev:
        res = hostlapack.bidiag_svd_many(
            [(vh[int(tab[r]["v_off"]):int(tab[r]["v_off"]) + int(tab[r]["n"])],
              vh[int(tab[r]["v_off"]) + int(tab[r]["n"]):int(tab[r]["v_off"]) + 2 * int(tab[r]["n"])])
             for r in range(len(on_dev))], lanes=_STEDC_LANES)
    sig = {}
    for r, i in enumerate(on_dev):
        sig[i] = np.maximum(res[r][0], 0.0)
    for i in off_dev:
        sig[i] = facs[i][3]
    kept = {}
    for it, (mt, blocks, chi, scale, normalize) in enumerate(items):
        ids = [i for i, s in enumerate(sec) if s[0] == it]
        cnt = _cut([sig[i] for i in ids], chi)[0]
        for j, i in enumerate(ids):
            kept[i] = int(cnt[j])
    # kept vectors of B: left (m rows, zero below n), right (n rows); two reflector sets each
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    chunk = 8 if sum((kept[i] + 7) // 8 for i in on_dev) * 2 >= 2 * n_sm else 2
    sets, items_q, zoff = [], [], {}
    z = 0
    for r, i in enumerate(on_dev):
        q = kept[i]
        if not q:
            continue
        mm, nn = int(tab[r]["m"]), int(tab[r]["n"])
        vo_r = int(tab[r]["v_off"])
        zl, zr = z, z + mm * q
        zoff[i] = (zl, zr)
        z += (mm + nn) * q
        sets.append((mm, nn, int(tab[r]["ul_off"]), vo_r + 2 * nn, zl, 0, 0))
        sets.append((nn, max(nn - 2, 0), int(tab[r]["vr_off"]), vo_r + 3 * nn, zr, 1, 0))
        for sidx in (len(sets) - 2, len(sets) - 1):
            for c0 in range(0, q, chunk):
                items_q.append((sidx, c0, min(chunk, q - c0), 0))
    if z:
        ns = sum(kept[i] for i in on_dev)
        pin = _pinned(z + ns)
        hz = pin.numpy()
        hz[:z] = 0.0
        so = z
        for r, i in enumerate(on_dev):
            q = kept[i]
            if not q:
                continue
            mm, nn = int(tab[r]["m"]), int(tab[r]["n"])
            s_, Ub, VTb = res[r]
            zl, zr = zoff[i]
            hz[zl:zl + mm * q].reshape(q, mm)[:, :nn] = Ub[:, :q].T
            hz[zr:zr + nn * q].reshape(q, nn)[:] = VTb[:q, :]
            hz[so:so + q] = sig[i][:q]
            so += q
        up = torch.empty(z + ns, dtype=torch.float64, device=dev)
        up.copy_(pin[:z + ns], non_blocking=True)
        _PIN["done"] = torch.cuda.Event()
        _PIN["done"].record()
        if timing is not None:
            timing["host_ms"] = timing.get("host_ms", 0.0) + (time.perf_counter() - t_host) * 1e3
        Zd, S_all = up[:z], up[z:]
        st_h = np.asarray(sets, dtype=np.int64)
        st_arr = np.zeros(len(sets), dtype=REFL_SET)
        for f, name in enumerate(("rows", "nrefl", "r_off", "tau_off", "z_off", "shift", "pad")):
            st_arr[name] = st_h[:, f]
        st_d = torch.from_numpy(st_arr.view(np.uint8)).to(dev)
        it_d = torch.from_numpy(np.asarray(items_q, dtype=np.int32)).to(dev)
        keep += [st_d, it_d]
        mark("back0")
        _lib.check(lib.tnk_ormqr_batched_f64(st_d.data_ptr(), it_d.data_ptr(), len(items_q),
                                             int(st_arr["rows"].max()), RF.data_ptr(),
                                             vec.data_ptr(), Zd.data_ptr(), sp),
                   "tnk_ormqr_batched_f64")
        mark("back1")
    elif on_dev and timing is not None:
        timing["host_ms"] = timing.get("host_ms", 0.0) + (time.perf_counter() - t_host) * 1e3
    so = 0
    for r, i in enumerate(on_dev):
        _, _, M, tr, mm, nn = sec[i]
        q = kept[i]
        R, Cc = M.shape
        if not q:
            facs[i] = (M.new_zeros((R, 0)), M.new_zeros(0), M.new_zeros((0, Cc)), sig[i])
            continue
        zl, zr = zoff[i]
        Lq = Zd[zl:zl + mm * q].view(q, mm)        # row j: left singular vector j of A
        Rq = Zd[zr:zr + nn * q].view(q, nn)        # row j: right singular vector j of A
        S = S_all[so:so + q]
        so += q
        if not tr:          # A = M: U = Q_L U_B, V = Q_R V_B
            facs[i] = (Lq.mT, S, Rq, sig[i])
        else:               # A = M^T = U_A S V_A^T: M = V_A S U_A^T
            facs[i] = (Rq.mT, S, Lq, sig[i])
    out = []
    for it, (mt, blocks, chi, scale, normalize) in enumerate(items):
        ids = [i for i, s in enumerate(sec) if s[0] == it]
        out.append(_trunc_finish(mt, blocks, [facs[i] for i in ids], chi, scale, normalize))
    if timing is not None:
        mark("end")
        torch.cuda.synchronize(dev)
        span = lambda a, b: ev[a].elapsed_time(ev[b]) if a in ev and b in ev else 0.0
        for k, (a, b) in {"reduce_ms": ("red0", "red1"), "back_ms": ("back0", "back1"),
                          "total_ms": ("red0", "end")}.items():
            timing[k] = timing.get(k, 0.0) + span(a, b)
        timing["sectors"] = len(sec)
        timing["sectors_on_device"] = len(on_dev)
    return out


def truncated_svd(m: BlockTensor, chi: int, scale: str = "none", driver=None,
                  method: str = "svd", normalize: bool = True, host: str = "auto",
                  dtype=torch.float64, gram_qr: bool = False):
    """U, S, Vh, disc of a two-leg block matrix, keeping the `chi` largest singular values over
    all sectors. `scale` folds S into the kept factor ('right': rows of Vh, 'left': columns of U,
    'none'), with S normalised to unit norm first, as the sweep does (tnkit/_dmrg.py:705-714).
    With method='gram', `host` chooses where the sectors are factored: 'device' (below; what
    'auto' means for FP64 CUDA blocks with scale 'right' / 'left' where the device supports it),
    'auto' otherwise (split between cuSOLVER and host LAPACK by cost), 'never' (each sector on
    cuSOLVER) or 'always' (host LAPACK only). For scale
    'right' / 'left' the side the sweep keeps canonical (U / Vh) of a near-square sector comes
    straight from its own Gram matrix and the other is the exact projection, with S the square
    roots of the Gram eigenvalues; gram_qr=True keeps the reference's form (the smaller Gram
    matrix, then a QR) everywhere. dtype=float32
    factors the blocks in FP32 (results returned in FP64; a sector whose FP32 eigensolver does
    not converge is redone in FP64). Inside a DMRG sweep near convergence the FP32 Gram matrix
    loses the small singular values and the environments built on its factors drift, so the
    sweep driver does not use it.
    host='device': the device Gram route (_gram_device_many: the sectors' reductions to
    tridiagonal form and the back-transformation of the kept vectors on the GPU, only the
    tridiagonal eigenproblems on the host); FP64 CUDA blocks, scale as above. With
    method='svd', host 'auto' / 'device' takes the device exact route on FP64 CUDA blocks
    (_svd_device_many: bidiagonalisation and back-transformations on the GPU, the bidiagonal
    SVDs on the host), 'never' keeps torch.linalg.svd per sector.
    Returns U, S (device vector, normalised when scale != 'none'), Vh, disc (absolute)."""
    if host not in ("auto", "never", "always", "device"):
        raise ValueError("host must be 'auto', 'never', 'always' or 'device'")
    if chi < 1:
        raise ValueError(f"chi must be at least 1, got {chi}")
    real_cuda = m.data.is_cuda and m.data.dtype == torch.float64 and dtype == torch.float64
    if method == "svd" and host in ("auto", "device") and real_cuda and \
            (host == "device" or device_svd_available()):
        blocks = list(_blocks(m))
        if not blocks:
            raise ValueError("the matrix has no allowed blocks")
        return _svd_device_many([(m, blocks, chi, scale, normalize)])[0]
    if host == "auto" and method == "gram" and not gram_qr and real_cuda and \
            scale in ("right", "left") and device_gram_available():
        host = "device"
    if host == "device":
        if method != "gram" or gram_qr or not real_cuda:
            raise ValueError("host='device' is the FP64 Gram or exact route of a CUDA block "
                             "matrix")
        blocks = list(_blocks(m))
        if not blocks:
            raise ValueError("the matrix has no allowed blocks")
        return _gram_device_many([(m, blocks, chi, scale, normalize)])[0]
    lr, lc = m.layout.legs
    low = dtype == torch.float32 and m.data.dtype == torch.float64
    if low and method != "gram":
        raise ValueError("an FP32 truncation needs method='gram'")
    blocks = list(_blocks(BlockTensor(m.layout, m.data.float()) if low else m))
    if method == "gram":
        fn = _svd_gram_native if (m.data.is_cuda and m.data.dtype == torch.float64) \
            else (lambda M: tuple(_svd_gram(M)) + (None,))
    elif method == "svd":
        fn = lambda M: tuple(torch.linalg.svd(M, full_matrices=False, driver=driver)) + (None,)
    else:
        raise ValueError(f"unknown method {method!r}; expected 'svd' or 'gram'")
    mats = [M for _, _, M in blocks]
    if method == "gram" and not gram_qr and not low and scale in ("right", "left"):
        def pick(M, base):
            R, Cc = M.shape
            o = 1 if scale == "right" and R <= 1.25 * Cc else \
                2 if scale == "left" and Cc <= 1.25 * R else 0
            return (lambda X: base(X, o)) if o else base
    else:
        pick = lambda M, base: base
    if len(mats) > 1 and m.data.is_cuda:
        if method == "gram" and fn is _svd_gram_native and host != "never":
            blas = _host_blas()
            shapes = [tuple(M.shape) for M in mats]
            lanes = _assign_sectors(shapes, blas is not None) if host == "auto" else \
                _assign_sectors(shapes, True, gpu_ok=False)
            fns = [pick(M, _svd_gram_host if l >= 0 else _svd_gram_native)
                   for M, l in zip(mats, lanes)]
            if low:
                fns = [_with_fp64_fallback(f) for f in fns]
            if any(l >= 0 for l in lanes) and blas is not None:
                prev = blas[1]()
                blas[0](max(1, prev // _HOST_THREADS_DIV))
                try:
                    facs = _map_hybrid(fns, mats, lanes, m.data.device)
                finally:
                    blas[0](prev)
            elif any(l >= 0 for l in lanes):
                facs = _map_hybrid(fns, mats, lanes, m.data.device)
            else:
                facs = _concurrent().map(fns, mats, m.data.device)
        else:
            fn1 = _with_fp64_fallback(fn) if low else fn
            facs = _concurrent().map([pick(M, fn1) if fn is _svd_gram_native else fn1
                                      for M in mats], mats, m.data.device)
    else:
        fn1 = _with_fp64_fallback(fn) if low else fn
        facs = [(pick(M, fn1) if fn is _svd_gram_native else fn1)(M) for M in mats]
    if low:
        facs = [(U.double(), S.double(), Vh.double(), h) for U, S, Vh, h in facs]
    return _trunc_finish(m, blocks, facs, chi, scale, normalize)


def _gram_pick(scale: str):
    """The Gram factorisation per sector shape: the side the sweep keeps canonical straight from
    its own Gram matrix for near-square sectors (orth 1 / 2), else the reference's QR form."""
    def pick(M, base):
        R, Cc = M.shape
        o = 1 if scale == "right" and R <= 1.25 * Cc else \
            2 if scale == "left" and Cc <= 1.25 * R else 0
        return (lambda X: base(X, o)) if o else base
    return pick


def truncated_svd_many(items, driver=None, method: str = "svd", normalize: bool = True,
                       host: str = "auto"):
    """truncated_svd of several FP64 CUDA block matrices -- e.g. one bond of each of many
    chains -- given as [(m, chi, scale)], with the sectors of all of them factored in one
    concurrent pass (GPU sectors a stream each, with method='gram' the host LAPACK share
    assigned over all sectors together). Returns the list of (U, S, Vh, disc)."""
    if host not in ("auto", "never", "always", "device"):
        raise ValueError("host must be 'auto', 'never', 'always' or 'device'")
    if method not in ("svd", "gram"):
        raise ValueError(f"unknown method {method!r}; expected 'svd' or 'gram'")
    if method == "svd" and host in ("auto", "device") and \
            all(m.data.is_cuda and m.data.dtype == torch.float64 for m, _, _ in items) and \
            (host == "device" or device_svd_available()):
        dv = []
        for m, chi, scale in items:
            if chi < 1:
                raise ValueError(f"chi must be at least 1, got {chi}")
            blocks = list(_blocks(m))
            if not blocks:
                raise ValueError("the matrix has no allowed blocks")
            dv.append((m, blocks, chi, scale, normalize))
        return _svd_device_many(dv)
    if host == "auto" and method == "gram" and all(sc in ("right", "left") for _, _, sc in items) \
            and all(m.data.is_cuda and m.data.dtype == torch.float64 for m, _, _ in items) \
            and device_gram_available():
        host = "device"
    if host == "device":
        if method != "gram":
            raise ValueError("host='device' is the Gram route")
        dv = []
        for m, chi, scale in items:
            if chi < 1:
                raise ValueError(f"chi must be at least 1, got {chi}")
            if not (m.data.is_cuda and m.data.dtype == torch.float64):
                raise TypeError("truncated_svd_many takes FP64 CUDA block matrices")
            blocks = list(_blocks(m))
            if not blocks:
                raise ValueError("the matrix has no allowed blocks")
            dv.append((m, blocks, chi, scale, normalize))
        return _gram_device_many(dv)
    per, fns, mats, shapes = [], [], [], []
    for m, chi, scale in items:
        if chi < 1:
            raise ValueError(f"chi must be at least 1, got {chi}")
        if not (m.data.is_cuda and m.data.dtype == torch.float64):
            raise TypeError("truncated_svd_many takes FP64 CUDA block matrices")
        blocks = list(_blocks(m))
        per.append((m, chi, scale, blocks, len(mats)))
        for _, _, M in blocks:
            mats.append(M)
            shapes.append((tuple(M.shape), scale))
    if not mats:
        raise ValueError("the matrices have no allowed blocks")
    if method == "svd":
        fn = lambda M: tuple(torch.linalg.svd(M, full_matrices=False, driver=driver)) + (None,)
        facs = _concurrent().map([fn] * len(mats), mats, mats[0].device) if len(mats) > 1 \
            else [fn(M) for M in mats]
    else:
        blas = _host_blas() if host != "never" else None
        # host='always' factors every sector with host LAPACK whether or not the library's
        # thread control was found (as truncated_svd does); 'auto' needs that control to split
        sh = [s_ for s_, _ in shapes]
        lanes = (_assign_sectors(sh, True, gpu_ok=False) if host == "always" else
                 [-1] * len(mats) if blas is None else _assign_sectors(sh, True))
        fns = [_gram_pick(sc)(M, _svd_gram_host if l >= 0 else _svd_gram_native)
               if sc in ("right", "left") else (_svd_gram_host if l >= 0 else _svd_gram_native)
               for M, (_, sc), l in zip(mats, shapes, lanes)]
        on_host = any(l >= 0 for l in lanes)
        if on_host and blas is not None:
            prev = blas[1]()
            blas[0](max(1, prev // _HOST_THREADS_DIV))
            try:
                facs = _map_hybrid(fns, mats, lanes, mats[0].device)
            finally:
                blas[0](prev)
        elif on_host:
            facs = _map_hybrid(fns, mats, lanes, mats[0].device)
        elif len(mats) > 1:
            facs = _concurrent().map(fns, mats, mats[0].device)
        else:
            facs = [f(M) for f, M in zip(fns, mats)]
    return [_trunc_finish(m, blocks, facs[b:b + len(blocks)], chi, scale, normalize)
            for m, chi, scale, blocks, b in per]


def _cut(svals, chi: int):
    """The global cut over the sectors' singular values (each sector's descending): the chi
    largest in the stable order of (-sigma, position) (the reference's order,
    tnkit/blocks.py:1427). Returns (kept count per sector, the order over the concatenated
    values, the number kept)."""
    s_host = np.concatenate(svals) if svals else np.zeros(0)
    owner = np.concatenate([np.full(len(x), j) for j, x in enumerate(svals)]) if svals else \
        np.zeros(0, dtype=np.int64)
    order = np.lexsort((np.arange(s_host.size), -s_host))
    k = min(int(chi), s_host.size)
    return np.bincount(owner[order[:k]], minlength=len(svals)), order, k


def _trunc_finish(m: BlockTensor, blocks, facs, chi: int, scale: str, normalize: bool):
    """The global cut over all sectors' singular values (descending, stable: the reference's
    order, tnkit/blocks.py:1427), the new bond leg, S normalised and folded into the kept
    factor."""
    lr, lc = m.layout.legs
    parts = [(r, c, U, S, Vh) for (r, c, _), (U, S, Vh, _h) in zip(blocks, facs)]
    if not parts:
        raise ValueError("the matrix has no allowed blocks")
    # every sector's singular values on the host (the factors may hold only the kept ones)
    if all(f[3] is not None for f in facs):
        s_host = np.concatenate([f[3] for f in facs])
        lens = [len(f[3]) for f in facs]
    else:
        s_host = torch.cat([p[3] for p in parts]).cpu().numpy().astype(np.float64)
        lens = [len(p[3]) for p in parts]
    kept, order, k = _cut([s_host[a:a + n] for a, n in zip(np.cumsum([0] + lens[:-1]), lens)],
                          chi)
    disc = float(np.sum(s_host[order[k:]] ** 2))
    norm = float(np.sqrt(np.sum(s_host[order[:k]] ** 2))) or 1.0
    new = [(_row_label(lr, r), r, c, U[:, :n], S[:n], Vh[:n])
           for (r, c, U, S, Vh), n in zip(parts, kept.tolist()) if n]
    new.sort(key=lambda x: (x[0], x[1]))
    bond = Leg(tuple(x[0] for x in new), tuple(int(x[4].shape[0]) for x in new), 1)
    if scale != "none" and normalize:
        new = [(q, r, c, U, S / norm, Vh) for (q, r, c, U, S, Vh) in new]
    Ub, Vb = [], []
    for q, r, c, U, S, Vh in sorted(new, key=lambda x: x[1]):
        Ub.append((U * S[None, :] if scale == "left" else U).reshape(-1))
    for q, r, c, U, S, Vh in new:
        Vb.append((Vh * S[:, None] if scale == "right" else Vh).reshape(-1))
    S = torch.cat([x[4] for x in new])
    Ul = canonical((lr, bond.flip()), _zero_like(m.layout.charge))
    Vl = canonical((bond, lc), m.layout.charge)
    return (BlockTensor(Ul, torch.cat(Ub).contiguous()), S,
            BlockTensor(Vl, torch.cat(Vb).contiguous()), disc)


def _zero_like(q):
    return tuple(0 for _ in q) if isinstance(q, tuple) else 0


def lq(m: BlockTensor):
    """m = L Q per block, Q with orthonormal rows (the new bond labelled by the row charge)."""
    lr, lc = m.layout.legs
    blocks = list(_blocks(m))

    def fac(M):
        q, t = torch.linalg.qr(M.mH)
        return t.mH.contiguous(), q.mH.contiguous()
    mats = [M for _, _, M in blocks]
    facs = _concurrent().map(fac, mats, m.data.device) if len(mats) > 1 and m.data.is_cuda \
        else [fac(M) for M in mats]
    new = [(_row_label(lr, r), r, c, a, b) for (r, c, _), (a, b) in zip(blocks, facs)]
    new.sort(key=lambda x: x[0])
    bond = Leg(tuple(x[0] for x in new), tuple(int(x[3].shape[1]) for x in new), 1)
    A = torch.cat([a.reshape(-1) for _, _, _, a, _ in sorted(new, key=lambda x: x[1])])
    B = torch.cat([b.reshape(-1) for _, _, _, _, b in new])
    return (BlockTensor(canonical((lr, bond.flip()), _zero_like(m.layout.charge)), A),
            BlockTensor(canonical((bond, lc), m.layout.charge), B))


class Scalars:
    """Norms and scalings of flat device buffers through the library's reduction kernels."""

    def __init__(self, device):
        self.red = torch.empty(_lib.TNK_RED_ELEMS, dtype=torch.float64, device=device)
        self.sc = torch.zeros(4, dtype=torch.float64, device=device)
        self.lib = _lib.lib()

    def normalize_(self, x: torch.Tensor) -> torch.Tensor:
        sp = _lib.stream_ptr()
        r = torch.view_as_real(x).reshape(-1) if x.is_complex() else x
        _lib.check(self.lib.tnk_nrm2_f64(r.data_ptr(), r.numel(), self.sc.data_ptr(),
                                         self.red.data_ptr(), sp), "nrm2")
        _lib.check(self.lib.tnk_scale_div_f64(r.data_ptr(), r.data_ptr(), r.numel(),
                                              self.sc.data_ptr(), 1.0, sp), "scale_div")
        return x

    def norm(self, x: torch.Tensor) -> float:
        sp = _lib.stream_ptr()
        x = torch.view_as_real(x).reshape(-1) if x.is_complex() else x
        _lib.check(self.lib.tnk_nrm2_f64(x.data_ptr(), x.numel(), self.sc.data_ptr(),
                                         self.red.data_ptr(), sp), "nrm2")
        return float(self.sc[0].item())

    def residual(self, v: torch.Tensor, w: torch.Tensor):
        """(rayleigh quotient th, ||w - th v|| / ||v||) of real FP64 buffers with w = H v; w is
        overwritten by w - th v."""
        sp = _lib.stream_ptr()
        n = v.numel()
        _lib.check(self.lib.tnk_nrm2_f64(v.data_ptr(), n, self.sc.data_ptr(),
                                         self.red.data_ptr(), sp), "nrm2")
        _lib.check(self.lib.tnk_dot_f64(v.data_ptr(), w.data_ptr(), n, self.sc.data_ptr() + 8,
                                        self.red.data_ptr(), sp), "dot")
        nv, vw = (float(x) for x in self.sc[:2].tolist())
        th = vw / (nv * nv)
        _lib.check(self.lib.tnk_axpby_f64(v.data_ptr(), w.data_ptr(), n, None, -th, None, 1.0,
                                          sp), "axpby")
        return th, self.norm(w) / nv
