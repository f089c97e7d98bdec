"""Mixed-precision local solve: tensor-core matvecs for the bulk of Lanczos, FP64 polish.

The two-site H_eff is applied on the tcgen05 tensor cores (TF32 inputs, FP32 accumulation in
TMEM; by default each operand split into TF32 hi/lo parts, three MMAs per product, ~1e-6
relative). The tensor-core stage keeps its Krylov basis in FP32 -- the operator is no more
accurate than that, and FP32 Gram-Schmidt runs on the FP32 pipes at half the bytes -- with the
projected eigenproblem, norms and dot products accumulated in FP64; the polish stage is the FP64
(or float-float) Lanczos, as in the reference's `lanczos_ground_mixed`
(tnkit/eigensolver.py:677-725): stage 1 converges the Ritz residual with
the cheap matvec to `tol_lo` (or until the residual stops improving, the floor the TF32 operator
allows), stage 2 restarts FP64 Lanczos from that vector to `tol` (at most `polish` iterations
when given). The reference refuses this mode on block tensors (tnkit/_dmrg.py:531-532); here it
runs on the U(1) block layout.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _lib
from . import linalg as LA
from . import plan as P
from .lanczos import lanczos_ground_restart
from .layout import Layout
from .ops import _PLANS, _pack, _two_site_key, host_plan_two_site
from .tensor import BlockTensor


class TwoSiteOperatorTC:
    """H_eff of one bond on the tensor cores, as `op(x, out)` on FP64 canonical buffers."""

    def __init__(self, theta_layout: Layout, L: BlockTensor, W1: BlockTensor, W2: BlockTensor,
                 R: BlockTensor, passes: int = 3):
        key = _two_site_key(theta_layout, L, W1, W2, R)
        tc = _PLANS.get_or(("tc",) + key, lambda: P.HostPlanTC(
            host_plan_two_site(theta_layout, L, W1, W2, R), theta_layout, L.layout, R.layout))
        self._setup(tc, L.data, R.data, theta_layout.size, passes)

    @classmethod
    def from_host_plan(cls, hp, L_data: torch.Tensor, R_data: torch.Tensor, n: int,
                       passes: int = 3) -> "TwoSiteOperatorTC":
        """The tensor-core operator of any two-site three-stage plan `hp` (a HostPlan3 whose
        slot 0 is `L_data`, slot 2 `R_data` and slot 1 a vector of n entries), e.g. a batched
        plan over many chains' local problems."""
        self = cls.__new__(cls)
        self._setup(P.HostPlanTC(hp, None, None, None), L_data, R_data, n, passes)
        return self

    def _setup(self, tc, L_data: torch.Tensor, R_data: torch.Tensor, n: int, passes: int):
        if passes not in (1, 3, 4):
            raise ValueError("passes must be 1 (TF32), 3 (split TF32, parts staged) or 4 (split "
                             "TF32, parts formed in shared memory)")
        dev = L_data.device
        self.device = dev
        self.passes = passes
        self.host = tc
        self.macs = tc.macs
        self.n = n
        self.stage = torch.empty(2 * tc.stage_elems, dtype=torch.float32, device=dev)
        self.y32 = torch.empty(max(tc.y32_elems, 1), dtype=torch.float32, device=dev)
        self.err = torch.zeros(16, dtype=torch.int32, device=dev)
        lib = _lib.lib()
        desc = np.ascontiguousarray(tc.map_desc_box())
        nmaps = desc.shape[0]
        maps_host = np.zeros(max(nmaps, 1) * 128, np.uint8)
        _lib.check(lib.tnk_tc_encode_tmaps_box(self.stage.data_ptr(), desc.ctypes.data, nmaps,
                                               maps_host.ctypes.data), "tnk_tc_encode_tmaps")
        arrays = [maps_host, tc.cvt["T"], tc.cvt_items["T"], tc.t1, tc.s1, tc.tiles1, tc.t2,
                  tc.c2, tc.items2, tc.t3, tc.s3, tc.tiles3, tc.cvt["L"], tc.cvt_items["L"],
                  tc.cvt["R"], tc.cvt_items["R"]]
        self.buf, offs = _pack(arrays, dev)
        a = [self.buf.data_ptr() + o for o in offs]
        self.c = _lib.TcPlan(a[1], a[2], len(tc.cvt_items["T"]),
                             a[3], a[4], a[5], len(tc.tiles1),
                             a[6], a[7], a[8], len(tc.items2),
                             a[9], a[10], a[11], len(tc.tiles3),
                             a[0], self.stage.data_ptr(), tc.stage_elems,
                             self.y32.data_ptr(), self.err.data_ptr(), passes, tc.bn3)
        sp = _lib.stream_ptr()
        split = 1 if passes == 3 else 0
        _lib.check(lib.tnk_stage_f32(a[12], a[13], len(tc.cvt_items["L"]), L_data.data_ptr(),
                                     self.stage.data_ptr(), tc.stage_elems, split, sp),
                   "stage L")
        _lib.check(lib.tnk_stage_f32(a[14], a[15], len(tc.cvt_items["R"]), R_data.data_ptr(),
                                     self.stage.data_ptr(), tc.stage_elems, split, sp),
                   "stage R")
        self.L, self.R = L_data, R_data   # staged copies were taken; keep the sources alive
        self.calls = 0

    def __call__(self, x: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        y = torch.empty_like(x) if out is None else out
        _lib.check(_lib.lib().tnk_apply_two_site_tc(C.byref(self.c), x.data_ptr(), y.data_ptr(),
                                                    _lib.stream_ptr()), "tnk_apply_two_site_tc")
        self.calls += 1
        return y

    def check_device_error(self):
        """Raise if a kernel of this operator recorded a timed-out wait (reads one word)."""
        e = int(self.err[0].item())
        if e:
            raise _lib.TnkError(_lib.TNK_ERR_CUDA, "tcgen05 grouped GEMM",
                                f"a bounded wait timed out (code {e}); results are invalid")


class _F32Vectors:
    """An operator on FP64 vectors applied to FP32 vectors (conversions on the device around
    it), for the FP32 Krylov basis of the tensor-core stage."""

    def __init__(self, op, n: int, device):
        self.op = op
        self.xd = torch.empty(n, dtype=torch.float64, device=device)
        self.yd = torch.empty(n, dtype=torch.float64, device=device)

    @property
    def calls(self):
        return self.op.calls

    def __call__(self, x: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        self.xd.copy_(x)
        self.op(self.xd, self.yd)
        out.copy_(self.yd)
        return out


_SCAL = {}


def _scalars(device) -> LA.Scalars:
    key = str(device)
    if key not in _SCAL:
        _SCAL[key] = LA.Scalars(device)
    return _SCAL[key]


def _fp64_residual(op64, v: torch.Tensor):
    """(rayleigh quotient, residual norm) of v in FP64: one FP64 matvec, then the library's
    norm / dot / axpy kernels."""
    return _scalars(v.device).residual(v, op64(v))


def refine_ground(op64, op_lo, x: torch.Tensor, tol: float, outer: int = 3, inner: int = 24,
                  check: int = 8, inner_tol: float = 1e-3):
    """Polish an approximate lowest eigenvector of H by defect correction: every outer step
    computes the residual r = H x - theta x in high precision (one matvec of `op64`, FP64 or
    float-float, theta the Rayleigh quotient) and solves the Jacobi-Davidson correction
    equation (I - x x^T)(H - theta)(I - x x^T) t = -r, t orthogonal to x, approximately with
    the cheap operator `op_lo` (the tensor-core matvec, ~1e-6 relative) by conjugate gradients
    (the projected operator is positive definite on x's complement once theta is below the
    second eigenvalue), then x <- (x + t) / ||x + t||. The error the cheap operator leaves in t
    is ~ ||H - H_lo|| / gap of t, so each outer step gains ~5 orders of magnitude; the FP64
    residual decides when to stop (Jacobi-Davidson: Sleijpen and van der Vorst, SIAM J. Matrix
    Anal. Appl. 17 (1996) 401; mixed-precision refinement of eigenpairs in the same spirit).
    CG's scalars stay on the device; its residual is read every `check` steps.
    Returns (theta, x, info) with info['residual'] the last FP64 residual norm (x unit norm)."""
    x = x / torch.linalg.vector_norm(x)
    y = torch.empty_like(x)
    hi = lo = 0
    theta, rn = 0.0, float("inf")
    for it in range(outer + 1):
        op64(x, y)
        hi += 1
        th = torch.dot(x, y)
        r = y - th * x
        rn = float(torch.linalg.vector_norm(r))
        theta = float(th)
        if rn < tol or it == outer or not np.isfinite(rn):
            break
        # CG on the projected correction equation, every vector orthogonal to x
        t = torch.zeros_like(x)
        res = -r
        res -= torch.dot(x, res) * x
        p = res.clone()
        rr = torch.dot(res, res)
        q = torch.empty_like(x)
        for j in range(inner):
            op_lo(p, q)
            lo += 1
            q -= th * p
            q -= torch.dot(x, q) * x
            pq = torch.dot(p, q)
            alpha = rr / pq
            t += alpha * p
            res -= alpha * q
            rr_new = torch.dot(res, res)
            if (j + 1) % check == 0 and float(rr_new) ** 0.5 < inner_tol * rn:
                break
            p = res + (rr_new / rr) * p
            rr = rr_new
        x = x + t
        x = x / torch.linalg.vector_norm(x)
    return theta, x, {"residual": rn, "n_hi": hi, "n_lo": lo, "outer": it}


def mixed_ground(theta_layout: Layout, L: BlockTensor, W1: BlockTensor, W2: BlockTensor,
                 R: BlockTensor, op64, v0: torch.Tensor, tol: float = 1e-9,
                 max_iter: int = 200, m: int = 40, k: int = 10, tol_lo: float = 1e-4,
                 basis=None, counts=None, passes: int = 3, polish: Optional[int] = None,
                 switch: float = 10.0, tc_only: bool = False, polish_mode: str = "lanczos"):
    """Lowest eigenpair of H_eff: tensor-core Lanczos to tol_lo, then FP64 Lanczos to tol.

    The warm start's FP64 residual is checked first (one FP64 matvec): a start already within
    `switch` * tol_lo of convergence -- late sweeps -- goes straight to the FP64 solve, which
    needs few iterations there and which the tensor-core operator (relative accuracy ~1e-6)
    could not improve; a start farther out -- the opening sweeps, bond growth -- spends its
    many iterations on the tensor cores.

    tc_only=True runs the tensor-core stage alone (to tol_lo, or until its residual stalls) and
    returns its vector: the local solve of the opening sweeps of the 'sweep' schedule.

    polish_mode='refine' polishes by defect correction (refine_ground: FP64 residuals,
    tensor-core correction solves) before any high-precision Lanczos, which then runs only if
    the residual is still above `tol` (and starts from the refined vector)."""
    if polish_mode not in ("lanczos", "refine"):
        raise ValueError("polish_mode must be 'lanczos' or 'refine'")
    if tc_only:
        op_lo = TwoSiteOperatorTC(theta_layout, L, W1, W2, R, passes=passes)
        e_lo, x32, info_lo = lanczos_ground_restart(
            _F32Vectors(op_lo, v0.numel(), v0.device), v0, tol=tol_lo, max_iter=max_iter, m=m,
            k=k, basis=basis, stall=8, dtype=torch.float32)
        op_lo.check_device_error()
        if counts is not None:
            counts["lo"] = counts.get("lo", 0) + op_lo.calls
        x = _scalars(x32.device).normalize_(x32.double())
        return e_lo, x, {"iters": info_lo["iters"], "converged": info_lo["converged"],
                         "e_lo": e_lo, "n_lo": op_lo.calls, "n_hi": 0, "matvecs": op_lo.calls}
    c0 = getattr(op64, "calls", 0)
    th0, r0 = _fp64_residual(op64, v0)
    n_lo = 0
    e_lo = th0
    x = v0
    if r0 < tol:
        e, info_hi = th0, {"iters": 0, "converged": True}
        x = _scalars(v0.device).normalize_(v0.clone())
    else:
        op_lo = None
        if r0 >= switch * tol_lo or polish_mode == "refine":
            op_lo = TwoSiteOperatorTC(theta_layout, L, W1, W2, R, passes=passes)
        if r0 >= switch * tol_lo:
            e_lo, x32, info_lo = lanczos_ground_restart(
                _F32Vectors(op_lo, v0.numel(), v0.device), v0, tol=max(tol_lo, tol),
                max_iter=max_iter, m=m, k=k, basis=basis, stall=8, dtype=torch.float32)
            op_lo.check_device_error()
            x = x32.double()
        info_hi = None
        if polish_mode == "refine":
            e, x, rinfo = refine_ground(op64, op_lo, x, tol)
            op_lo.check_device_error()
            if rinfo["residual"] < tol:
                info_hi = {"iters": rinfo["outer"], "converged": True}
        if info_hi is None:
            e, x, info_hi = lanczos_ground_restart(op64, x, tol=tol,
                                                   max_iter=max_iter if polish is None
                                                   else polish, m=m, k=k, basis=basis)
        n_lo = 0 if op_lo is None else op_lo.calls
    n_hi = getattr(op64, "calls", 0) - c0
    if counts is not None:
        counts["lo"] = counts.get("lo", 0) + n_lo
        counts["hi"] = counts.get("hi", 0) + n_hi
    return e, x, {"iters": info_hi["iters"], "converged": info_hi["converged"], "e_lo": e_lo,
                  "r0": r0, "n_lo": n_lo, "n_hi": n_hi, "matvecs": n_lo + n_hi}
