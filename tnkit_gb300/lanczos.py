"""Thick-restart Lanczos on the GPU (tnkit/eigensolver.py:507-674).

The Krylov basis (m+1 vectors) lives on the device. One iteration is the matvec and three fused
classical Gram-Schmidt launches (tnk_cgs_pass_f64): c1 = V^T w; w -= V c1 with c2 = V^T w in the
same read of V; w -= V c2 with beta = ||w|| in the same read -- the reference's CGS2
(tnkit/eigensolver.py:581-595), which also removes the three-term and arrowhead couplings the
reference subtracts first, with alpha = <v_j, H v_j> = c1[j]. Every reduction is deterministic
and finishes inside its launch; the coefficients and beta land in a device record that one
asynchronous copy brings to pinned host memory.

The host solves the projected (<= m x m) eigenproblem with LAPACK, as the reference does
(a tridiagonal solver for the lowest pair before the first restart, the full symmetric one after).
Its work overlaps the GPU: the next iteration, which needs nothing from the host, is queued before
the host waits for the current one, unless the residual trend says the current one is likely the
last; a queued iteration that turns out not to be needed is discarded (it writes only the next
basis row and the work vector). The restart's basis rotation is one grouped-GEMM launch.

The algorithm, stopping rule (Ritz residual |beta * y_last| < tol), breakdown rule
(beta < 1e-12 max(1, |alpha|)) and restart (k lowest Ritz vectors plus the residual direction,
arrowhead projected matrix) are the reference's.
"""
from __future__ import annotations

from typing import Callable, Optional

import numpy as np
import torch
from scipy.linalg import eigh_tridiagonal

from . import _lib
from ._lib import GEMM_SEG, GEMM_TASK, GEMM_TILE
from .plan import TILE_M, TILE_N

_MAXNV = 64
_REC = 1 + 2 * _MAXNV           # per-iteration device record: beta, c1[0:64], c2[0:64]
_SUB, _DOT, _NRM = 1, 2, 4      # tnk_cgs_pass_f64 modes


class _Dev:
    """Device scratch of one solve: reduction workspace and completion counter, scalar slots,
    two iteration records (device and pinned host, alternating) with their events."""

    def __init__(self, device, dtype=torch.float64):
        self.f32 = dtype == torch.float32
        self.red = torch.empty(_lib.TNK_RED_ELEMS, dtype=torch.float64, device=device)
        self.cnt = torch.zeros(4, dtype=torch.int32, device=device)
        self.sc = torch.zeros(8 + _MAXNV, dtype=torch.float64, device=device)
        self.host = torch.zeros(8, dtype=torch.float64, pin_memory=True)
        self.rec = torch.zeros((2, _REC), dtype=torch.float64, device=device)
        self.hrec = torch.zeros((2, _REC), dtype=torch.float64, pin_memory=True)
        self.ev = [torch.cuda.Event(), torch.cuda.Event()]
        self.lib = _lib.lib()
        self.sp = _lib.stream_ptr()

    def addr(self, i):
        return self.sc.data_ptr() + 8 * i

    def raddr(self, par, i):
        return self.rec.data_ptr() + 8 * (par * _REC + i)

    def nrm2(self, x, slot):
        if x.dtype == torch.float32:
            _lib.check(self.lib.tnk_cgs_pass_f32(None, x.numel(), 0, None, x.data_ptr(),
                                                 x.numel(), self.addr(slot), _NRM,
                                                 self.red.data_ptr(), self.cnt.data_ptr(),
                                                 self.sp), "nrm2")
            return
        _lib.check(self.lib.tnk_nrm2_f64(x.data_ptr(), x.numel(), self.addr(slot),
                                         self.red.data_ptr(), self.sp), "nrm2")

    def scale_div(self, x, y, s_addr, f=1.0):
        fn = self.lib.tnk_scale_div_f32 if x.dtype == torch.float32 else \
            self.lib.tnk_scale_div_f64
        _lib.check(fn(x.data_ptr(), y.data_ptr(), x.numel(), s_addr, f, self.sp), "scale_div")

    def cgs(self, V, nv, cin, w, out, mode):
        fn = self.lib.tnk_cgs_pass_f32 if self.f32 else self.lib.tnk_cgs_pass_f64
        _lib.check(fn(V.data_ptr(), V.stride(0), nv, cin, w.data_ptr(), w.numel(), out, mode,
                      self.red.data_ptr(), self.cnt.data_ptr(), self.sp), "cgs_pass")

    def gemv_sub(self, V, nv, w):
        """w -= V[:nv]^T c with c in the coefficient slots (set_coeffs)."""
        self.cgs(V, nv, self.addr(8), w, None, _SUB)

    def set_coeffs(self, c: np.ndarray):
        self.sc[8:8 + len(c)].copy_(torch.as_tensor(np.ascontiguousarray(c, np.float64)))

    def read_slot(self, i):
        self.host[i:i + 1].copy_(self.sc[i:i + 1], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return float(self.host[i])

    def issue(self, matvec, V, w, j, count, scale):
        """Queue iteration `count` (basis row j): [V[j] = w / beta of the previous iteration],
        w = H V[j], CGS2 against V[0..j], beta; then the record's copy to the host and its event.
        Returns the record parity."""
        par = count & 1
        if scale:
            self.scale_div(w, V[j], self.raddr(par ^ 1, 0))
        matvec(V[j], w)
        nv = j + 1
        c1, c2 = self.raddr(par, 1), self.raddr(par, 1 + _MAXNV)
        self.cgs(V, nv, None, w, c1, _DOT)
        self.cgs(V, nv, c1, w, c2, _SUB | _DOT)
        self.cgs(V, nv, c2, w, self.raddr(par, 0), _SUB | _NRM)
        self.hrec[par].copy_(self.rec[par], non_blocking=True)
        self.ev[par].record()
        return par

    def wait(self, par, j):
        """(alpha, beta) of the iteration recorded in `par` (basis row j)."""
        self.ev[par].synchronize()
        h = self.hrec[par]
        return float(h[1 + j]), float(h[0])

    def rotate(self, Y: np.ndarray, V: torch.Tensor, out: torch.Tensor):
        """out (kk x n) = Y^T (kk x cur) @ V[:cur] as one grouped-GEMM launch (FP64), or one
        tnk_rotate_f32 launch for an FP32 basis."""
        cur, kk = Y.shape
        n = V.shape[1]
        if V.dtype == torch.float32:
            Yd = torch.as_tensor(np.ascontiguousarray(Y, dtype=np.float64), device=V.device)
            _lib.check(self.lib.tnk_rotate_f32(V.data_ptr(), V.stride(0), cur, Yd.data_ptr(), kk,
                                               out.data_ptr(), out.stride(0), n, self.sp),
                       "rotate")
            return (Yd,)
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


def _lowest(T: np.ndarray, cur: int, tridiagonal: bool):
    """Lowest eigenpair of the projected matrix T[:cur, :cur]."""
    if cur == 1:
        return float(T[0, 0]), np.array([1.0])
    if tridiagonal:
        ev, evec = eigh_tridiagonal(np.diagonal(T)[:cur].copy(),
                                    np.diagonal(T, 1)[:cur - 1].copy(), select="i",
                                    select_range=(0, 0), check_finite=False)
    else:
        ev, evec = np.linalg.eigh(T[:cur, :cur])
    return float(ev[0]), evec[:, 0]


def lanczos_ground_restart(matvec: Callable, v0: torch.Tensor, tol: float = 1e-8,
                           max_iter: int = 200, m: int = 40, k: int = 10,
                           basis: Optional[torch.Tensor] = None, stall: int = 0,
                           speculate: bool = True, dtype=torch.float64):
    """Lowest eigenpair of the operator `matvec(x, out) -> out` from the start `v0` (float64
    CUDA vector). Returns (theta, x, info) like the reference; x is normalised.

    stall > 0 also stops when the Ritz residual has improved by less than 10 % over the last
    `stall` iterations (info["stalled"]): the floor of a low-precision operator.
    speculate=False waits for every iteration before queuing the next (no discarded matvec).
    dtype=torch.float32 keeps the Krylov basis, the operator's vectors and x in FP32 (for an
    operator that is itself only FP32-accurate); the scalars stay FP64."""
    if k >= m:
        k = max(1, m // 2)
    if m + 1 > _MAXNV:
        raise ValueError(f"restart window m={m} exceeds {_MAXNV - 1}")
    if max_iter < 1:
        raise ValueError("max_iter must be >= 1")
    if dtype not in (torch.float64, torch.float32):
        raise ValueError("dtype must be torch.float64 or torch.float32")
    dev = v0.device
    D = _Dev(dev, dtype)
    n = v0.numel()
    v0 = v0.reshape(-1)
    D.nrm2(v0, 2)
    n0 = D.read_slot(2)
    if not np.isfinite(n0) or n0 < 1e-300:
        return 0.0, v0.to(dtype), {"iters": 0, "converged": False, "restarts": 0, "matvecs": 0}
    if basis is not None and basis.dtype != dtype:
        flat = basis.reshape(-1).view(dtype)         # the same storage, reinterpreted
        basis = flat[:(m + 1) * n].view(m + 1, n) if flat.numel() >= (m + 1) * n else None
    Vb = basis if (basis is not None and basis.shape[0] >= m + 1 and basis.shape[1] == n) \
        else torch.empty((m + 1, n), dtype=dtype, device=dev)
    if dtype == torch.float64:
        D.scale_div(v0, Vb[0], D.addr(2))
    else:
        Vb[0].copy_(v0)
        D.scale_div(Vb[0], Vb[0], D.addr(2))
    w = torch.empty(n, dtype=dtype, device=dev)
    T = np.zeros((m + 1, m + 1))
    n_kept = 0
    theta, y = 0.0, np.array([1.0])
    converged, stalled, restarts, it = False, False, 0, 0
    keep = []
    hist = []
    res = None
    issued = 1
    pending = [(0, D.issue(matvec, Vb, w, 0, 0, scale=False))]

    def likely_last():
        # the iteration being waited for converges if its residual falls below tol: predict it
        # from the last two residuals (geometric trend) and skip queuing past it when it would
        if len(hist) < 2 or hist[-2] <= 0.0:
            return False
        q = min(1.0, hist[-1] / hist[-2])
        return hist[-1] * q < 10.0 * tol

    while True:
        j, par = pending.pop(0)
        if (speculate and not pending and j + 1 < m and it + 1 < max_iter
                and not likely_last()):
            pending.append((j + 1, D.issue(matvec, Vb, w, j + 1, issued, scale=True)))
            issued += 1
        alpha, beta = D.wait(par, j)
        T[j, j] = alpha
        cur = j + 1
        th, y = _lowest(T, cur, n_kept == 0)
        it += 1
        res = abs(beta) * abs(float(y[-1]))
        hist.append(res)
        breakdown = (not np.isfinite(beta) or not np.isfinite(alpha)
                     or beta < 1e-12 * max(1.0, abs(alpha)))
        theta = th
        if breakdown or res < tol:
            converged = True
            break
        if stall and len(hist) > stall and res > 0.9 * hist[-stall - 1]:
            stalled = True
            break
        if it >= max_iter:
            break
        if cur >= m:                                 # thick restart (nothing queued here)
            ev, evec = np.linalg.eigh(T[:cur, :cur])
            kk = min(k, cur - 1)
            Yk = evec[:, :kk]
            tmp = torch.empty((kk, n), dtype=dtype, device=dev)
            keep = D.rotate(Yk, Vb[:cur], tmp)
            Vb[:kk].copy_(tmp)
            T[:] = 0.0
            border = beta * np.asarray(Yk[cur - 1, :], dtype=np.float64)
            for i in range(kk):
                T[i, i] = ev[i]
                T[i, kk] = T[kk, i] = border[i]
            n_kept = kk
            y = np.zeros(kk + 1)
            y[0] = 1.0
            restarts += 1
            pending.append((kk, D.issue(matvec, Vb, w, kk, issued, scale=True)))
            issued += 1
            continue
        T[j, j + 1] = T[j + 1, j] = beta
        if not pending:
            pending.append((j + 1, D.issue(matvec, Vb, w, j + 1, issued, scale=True)))
            issued += 1
    ny = len(y)
    x = torch.zeros(n, dtype=dtype, device=dev)
    D.set_coeffs(-np.asarray(y[:ny], np.float64))
    D.gemv_sub(Vb, ny, x)
    D.nrm2(x, 3)
    D.scale_div(x, x, D.addr(3))
    del keep
    return theta, x, {"iters": it, "converged": converged, "restarts": restarts,
                      "stalled": stalled, "residual": res, "matvecs": issued,
                      "discarded": issued - it}
