"""Thick-restart Lanczos on the GPU (tnkit/eigensolver.py:507-674).

The Krylov basis (m+1 vectors) lives on the device; every vector operation is a tnk_* kernel:
alpha = <v, w> and beta = ||w|| as deterministic two-phase reductions, the two classical
Gram-Schmidt passes as one multi-dot plus one GEMV each, the three-term and arrowhead couplings
as axpy/GEMV with their scalars read from device memory. The host reads two doubles per
iteration (alpha, beta) for the projected (m x m) eigenproblem, which it solves with LAPACK, as
the reference does; the restart's basis rotation is one grouped-GEMM launch.

The algorithm, stopping rule (Ritz residual |beta * y_last| < tol), breakdown rule
(beta < 1e-12 max(1, |alpha|)) and restart (k lowest Ritz vectors plus the residual direction,
arrowhead projected matrix) are the reference's.
"""
from __future__ import annotations

import ctypes as C
import time
from typing import Callable, Optional

import numpy as np
import torch

from . import _lib
from ._lib import GEMM_SEG, GEMM_TASK, GEMM_TILE
from .plan import TILE_M, TILE_N

_MAXNV = 64


class _Dev:
    """Device scratch of one solve: reduction workspace, scalar slots and a pinned mirror."""

    def __init__(self, device):
        self.red = torch.empty(_lib.TNK_RED_ELEMS, dtype=torch.float64, device=device)
        self.sc = torch.zeros(8 + _MAXNV, dtype=torch.float64, device=device)
        self.host = torch.zeros(8, dtype=torch.float64, pin_memory=True)
        self.lib = _lib.lib()
        self.sp = _lib.stream_ptr()

    def addr(self, i):
        return self.sc.data_ptr() + 8 * i

    def nrm2(self, x, slot):
        _lib.check(self.lib.tnk_nrm2_f64(x.data_ptr(), x.numel(), self.addr(slot),
                                         self.red.data_ptr(), self.sp), "nrm2")

    def dot(self, x, y, slot):
        _lib.check(self.lib.tnk_dot_f64(x.data_ptr(), y.data_ptr(), x.numel(), self.addr(slot),
                                        self.red.data_ptr(), self.sp), "dot")

    def axpby(self, x, y, fa, fb, sa=None, sb=None):
        _lib.check(self.lib.tnk_axpby_f64(x.data_ptr(), y.data_ptr(), x.numel(),
                                          None if sa is None else self.addr(sa), fa,
                                          None if sb is None else self.addr(sb), fb, self.sp),
                   "axpby")

    def scale_div(self, x, y, slot, f=1.0):
        _lib.check(self.lib.tnk_scale_div_f64(x.data_ptr(), y.data_ptr(), x.numel(),
                                              self.addr(slot), f, self.sp), "scale_div")

    def multidot(self, V, nv, w):
        n = w.numel()
        _lib.check(self.lib.tnk_multidot_f64(V.data_ptr(), V.stride(0), nv, w.data_ptr(), n,
                                             self.addr(8), self.red.data_ptr(), self.sp),
                   "multidot")

    def gemv_sub(self, V, nv, w):
        _lib.check(self.lib.tnk_gemv_sub_f64(V.data_ptr(), V.stride(0), nv, self.addr(8),
                                             w.data_ptr(), w.numel(), self.sp), "gemv_sub")

    def set_coeffs(self, c: np.ndarray):
        self.sc[8:8 + len(c)].copy_(torch.as_tensor(np.ascontiguousarray(c, np.float64)))

    def read(self, n=2):
        self.host[:n].copy_(self.sc[:n], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return self.host[:n].tolist()

    def rotate(self, Y: np.ndarray, V: torch.Tensor, out: torch.Tensor):
        """out (kk x n) = Y^T (kk x cur) @ V[:cur] as one grouped-GEMM launch."""
        cur, kk = Y.shape
        n = V.shape[1]
        A = torch.as_tensor(np.ascontiguousarray(Y.T), dtype=torch.float64, device=V.device)
        task = np.array([(0, n, kk, n, 0, 1, 0)], dtype=GEMM_TASK)
        seg = np.array([(0, 0, cur, 1, V.stride(0), 1, cur, 0, 1, 0, 0, 1.0)], dtype=GEMM_SEG)
        n0 = np.arange(0, n, TILE_N, dtype=np.int32)
        m0 = np.arange(0, kk, TILE_M, dtype=np.int32)
        tl = np.zeros(len(n0) * len(m0), dtype=GEMM_TILE)
        tl["m0"] = np.repeat(m0, len(n0))
        tl["n0"] = np.tile(n0, len(m0))
        dev = V.device
        t_task = torch.from_numpy(task.view(np.uint8).copy()).to(dev)
        t_seg = torch.from_numpy(seg.view(np.uint8).copy()).to(dev)
        t_tl = torch.from_numpy(tl.view(np.uint8).copy()).to(dev)
        _lib.check(self.lib.tnk_grouped_gemm_f64(t_task.data_ptr(), t_seg.data_ptr(),
                                                 t_tl.data_ptr(), len(tl), A.data_ptr(),
                                                 V.data_ptr(), 0, 0, out.data_ptr(), self.sp),
                   "rotate")
        return A, t_task, t_seg, t_tl       # keep alive until the stream passes them


def lanczos_ground_restart(matvec: Callable, v0: torch.Tensor, tol: float = 1e-8,
                           max_iter: int = 200, m: int = 40, k: int = 10,
                           timers: Optional[dict] = None, basis: Optional[torch.Tensor] = None,
                           stall: int = 0):
    """Lowest eigenpair of the operator `matvec(x, out) -> out` from the start `v0` (float64
    CUDA vector). Returns (theta, x, info) like the reference; x is normalised.

    stall > 0 also stops when the Ritz residual has improved by less than 10 % over the last
    `stall` iterations (info["stalled"]): the floor of a low-precision operator."""
    if k >= m:
        k = max(1, m // 2)
    if m + 1 > _MAXNV:
        raise ValueError(f"restart window m={m} exceeds {_MAXNV - 1}")
    dev = v0.device
    D = _Dev(dev)
    n = v0.numel()
    v0 = v0.reshape(-1)
    D.nrm2(v0, 2)
    D.host[2:3].copy_(D.sc[2:3], non_blocking=True)
    torch.cuda.current_stream().synchronize()
    n0 = float(D.host[2])
    if not np.isfinite(n0) or n0 < 1e-300:
        return 0.0, v0, {"iters": 0, "converged": False, "restarts": 0}
    Vb = basis if (basis is not None and basis.shape[0] >= m + 1 and basis.shape[1] == n) \
        else torch.empty((m + 1, n), dtype=torch.float64, device=dev)
    D.scale_div(v0, Vb[0], 2)
    w = torch.empty(n, dtype=torch.float64, device=dev)
    T = np.zeros((m + 1, m + 1))
    nV, n_kept, border = 1, 0, None
    beta_prev, v_prev = 0.0, None
    theta, y = 0.0, np.array([1.0])
    converged, restarts, it, j = False, 0, 0, 0
    keep = []
    hist = []
    stalled = False
    tm = timers if timers is not None else None
    while it < max_iter:
        t0 = time.perf_counter() if tm is not None else 0.0
        v = Vb[j]
        matvec(v, w)
        if n_kept and j == n_kept:
            D.set_coeffs(border)
            D.gemv_sub(Vb, n_kept, w)
        elif j > 0:
            D.axpby(v_prev, w, -beta_prev, 1.0)
        D.dot(v, w, 0)
        D.axpby(v, w, -1.0, 1.0, sa=0)
        for _ in range(2):
            D.multidot(Vb, nV, w)
            D.gemv_sub(Vb, nV, w)
        D.nrm2(w, 1)
        alpha, beta = D.read(2)
        if tm is not None:
            tm["device"] = tm.get("device", 0.0) + time.perf_counter() - t0
        T[j, j] = alpha
        cur = j + 1
        if cur == 1:
            th, y = alpha, np.array([1.0])
        else:
            ev, evec = np.linalg.eigh(T[:cur, :cur])
            th, y = float(ev[0]), evec[:, 0]
        it += 1
        res = abs(beta) * abs(float(y[-1]))
        breakdown = (not np.isfinite(beta) or not np.isfinite(alpha)
                     or beta < 1e-12 * max(1.0, abs(alpha)))
        theta = th
        if breakdown or res < tol:
            converged = True
            break
        if stall:
            hist.append(res)
            if len(hist) > stall and res > 0.9 * hist[-stall - 1]:
                stalled = True
                break
        if cur >= m:                                 # thick restart
            ev, evec = np.linalg.eigh(T[:cur, :cur])
            kk = min(k, cur - 1)
            Yk = evec[:, :kk]
            tmp = torch.empty((kk, n), dtype=torch.float64, device=dev)
            keep = D.rotate(Yk, Vb[:cur], tmp)
            D.axpby(tmp.reshape(-1), Vb[:kk].reshape(-1), 1.0, 0.0)
            D.scale_div(w, Vb[kk], 1)
            nV = kk + 1
            T[:] = 0.0
            border = beta * np.asarray(Yk[cur - 1, :], dtype=np.float64)
            for i in range(kk):
                T[i, i] = ev[i]
                T[i, kk] = T[kk, i] = border[i]
            n_kept, j = kk, kk
            beta_prev, v_prev = 0.0, None
            y = np.zeros(kk + 1)
            y[0] = 1.0
            restarts += 1
            continue
        T[j, j + 1] = T[j + 1, j] = beta
        v_prev, beta_prev = v, beta
        D.scale_div(w, Vb[j + 1], 1)
        nV = j + 2
        j += 1
    ny = min(len(y), nV)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    D.set_coeffs(-np.asarray(y[:ny], np.float64))
    D.gemv_sub(Vb, ny, x)
    D.nrm2(x, 3)
    D.scale_div(x, x, 3)
    del keep
    return theta, x, {"iters": it, "converged": converged, "restarts": restarts,
                      "stalled": stalled, "residual": res if it else None}
