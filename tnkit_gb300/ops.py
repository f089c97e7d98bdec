"""Device execution of the planned contractions through the C ABI.

`DevicePlan3` uploads a host plan's tables to the GPU once (one byte buffer, 64-byte aligned
sections) and launches the three stages with `tnk_*_f64`. The hot-path functions below mirror
the reference's tnkit/_dmrg.py:162-231 signatures on `BlockTensor` operands and cache their
plans per (layouts, MPO tensors). There is no fallback: without the library or a CUDA device they
raise.
"""
from __future__ import annotations

import ctypes as C
import threading
from collections import OrderedDict
from typing import Dict, Optional

import numpy as np
import torch

from . import _lib
from . import plan as P
from .layout import Layout
from .tensor import BlockTensor

_ALIGN = 64


def _require_cuda(*ts):
    """All operands contiguous CUDA float64, or all complex128; returns True when complex."""
    kinds = set()
    for t in ts:
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous()
                and t.dtype in (torch.float64, torch.complex128)):
            raise TypeError("tnkit_gb300 kernels need contiguous float64 or complex128 CUDA "
                            "tensors")
        kinds.add(t.dtype)
    if len(kinds) > 1:
        raise TypeError("tnkit_gb300 kernels need operands of one dtype (float64 or "
                        "complex128); cast the state with .to(torch.complex128) first")
    return torch.complex128 in kinds


def _cplx(hp):
    return P.ComplexPlan3(hp)


def _pack(arrays, device):
    """Concatenate numpy arrays into one device byte buffer; return (buffer, byte offsets).
    The bytes are staged in pinned host memory and copied without waiting for the stream, so
    building a plan never drains the GPU's queue (the caching host allocator keeps the staging
    block until the copy has run)."""
    offs, total = [], 0
    for a in arrays:
        offs.append(total)
        total += (a.nbytes + _ALIGN - 1) // _ALIGN * _ALIGN
    total = max(total, _ALIGN)
    dev = torch.device(device)
    pinned = dev.type == "cuda"
    host_t = torch.empty(total, dtype=torch.uint8, pin_memory=pinned)
    host = host_t.numpy()
    for a, o in zip(arrays, offs):
        if a.nbytes:
            host[o:o + a.nbytes] = np.frombuffer(np.ascontiguousarray(a).data, np.uint8)
    buf = host_t.to(dev, non_blocking=pinned)
    return buf, offs


class DevicePlan3:
    """A three-stage plan resident on the GPU. With ff=True its stage-1 tasks write float-float
    intermediates (flags bit 3), for the float-float entry points."""

    def __init__(self, hp: P.HostPlan3, device, ff: bool = False):
        self.host = hp
        (t1, s1, l1), (t2, c2, i2), (t3, s3, l3) = hp.g1, hp.c2, hp.g3
        t4, c4, i4 = hp.c4
        if ff:
            t1 = t1.copy()
            t1["flags"] |= 8
            for s in (s1, s3):
                if len(s) and not np.all(np.abs(s["coef"]) == 1.0):
                    raise ValueError("float-float plans need GEMM coefficients of +-1")
        arrays = [t1, s1, l1, t2, c2, i2, t3, s3, l3, t4, c4, i4]
        self.buf, offs = _pack(arrays, device)
        base = self.buf.data_ptr()
        a = [base + o for o in offs]
        out_elems = hp.out_layout.size * (2 if hp.kind.endswith("c128") else 1)
        self.out_elems = out_elems
        self.c = _lib.Plan3(a[0], a[1], a[2], len(l1), a[3], a[4], a[5], len(i2),
                            a[6], a[7], a[8], len(l3), hp.ws1, hp.ws2, out_elems,
                            a[9], a[10], a[11], len(i4))
        self.out_layout = hp.out_layout
        self.ws_elems = hp.ws_elems
        self.macs = hp.macs
        self.ref_macs = hp.ref_macs

    def run(self, fn: str, x0, x1, x2, out, ws, stream=None):
        lib = _lib.lib()
        if ws is None or ws.numel() < self.ws_elems:
            ws = workspace(self.ws_elems, out.device)
        f = getattr(lib, fn)
        sp = _lib.stream_ptr(stream)
        if fn in ("tnk_update_left_env_f64", "tnk_update_right_env_f64"):
            # (plan, env, site tensor, out, ws, n, stream): x0 = site tensor, x1 = env
            rc = f(C.byref(self.c), _lib.ptr(x1), _lib.ptr(x0), _lib.ptr(out), _lib.ptr(ws),
                   ws.numel(), sp)
        else:
            rc = f(C.byref(self.c), _lib.ptr(x0), _lib.ptr(x1), _lib.ptr(x2), _lib.ptr(out),
                   _lib.ptr(ws), ws.numel(), sp)
        _lib.check(rc, fn)
        return out


class DeviceGemmPlan:
    def __init__(self, hp: P.HostGemmPlan, device):
        self.host = hp
        t, s, l = hp.g
        self.buf, offs = _pack([t, s, l], device)
        base = self.buf.data_ptr()
        self.ptrs = [base + o for o in offs]
        self.n_tiles = len(l)
        self.out_layout = hp.out_layout
        self.macs = hp.macs

    def run(self, a, b, out, stream=None):
        rc = _lib.lib().tnk_grouped_gemm_f64(self.ptrs[0], self.ptrs[1], self.ptrs[2],
                                             self.n_tiles, _lib.ptr(a), _lib.ptr(b), 0, 0,
                                             _lib.ptr(out), _lib.stream_ptr(stream))
        _lib.check(rc, "tnk_grouped_gemm_f64")
        return out


class DeviceCombPlan:
    def __init__(self, hp: P.HostCombPlan, device):
        self.host = hp
        t, u, i = hp.c
        self.buf, offs = _pack([t, u, i], device)
        base = self.buf.data_ptr()
        self.ptrs = [base + o for o in offs]
        self.n_items = len(i)
        self.out_layout = hp.out_layout

    def run(self, src, dst, stream=None):
        rc = _lib.lib().tnk_combine_f64(self.ptrs[0], self.ptrs[1], self.ptrs[2], self.n_items,
                                        _lib.ptr(src), _lib.ptr(dst), _lib.stream_ptr(stream))
        _lib.check(rc, "tnk_combine_f64")
        return dst


# --------------------------------------------------------------------------- #
# workspace and plan caches
# --------------------------------------------------------------------------- #
_WS: Dict[tuple, torch.Tensor] = {}


def workspace(n: int, device) -> torch.Tensor:
    """A grow-only float64 workspace per device and current stream (that stream orders its
    reuse; work on another stream, e.g. another thread's, gets its own)."""
    device = torch.device(device)
    key = (device, torch.cuda.current_stream(device).cuda_stream if device.type == "cuda"
           else 0)
    w = _WS.get(key)
    if w is None or w.numel() < n:
        w = torch.empty(max(n, 1 << 16), dtype=torch.float64, device=device)
        _WS[key] = w
    return w


class _LRU(OrderedDict):
    """Bounded cache of plans; safe to share between host threads (a plan may be built twice
    when two threads miss at once, and the first stored wins)."""

    def __init__(self, cap):
        super().__init__()
        self.cap = cap
        self._lock = threading.Lock()

    def get_or(self, key, build):
        with self._lock:
            v = self.get(key)
            if v is not None:
                self.move_to_end(key)
                return v
        v = build()
        with self._lock:
            old = self.get(key)
            if old is not None:
                return old
            self[key] = v
            while len(self) > self.cap:
                self.popitem(last=False)
        return v


_PLANS = _LRU(2048)


def _mpo_key(W: BlockTensor):
    # MPO tensors are fixed per site: identity plus the object itself keeps it alive in the key
    return (id(W), W)


def _host_of(W: BlockTensor) -> np.ndarray:
    if W.host is None:
        W.host = W.data.detach().cpu().numpy()
    return W.host


def _real_plan(key, build):
    return _PLANS.get_or(("host",) + key, build)


def _two_site_key(theta: Layout, L: BlockTensor, W1: BlockTensor, W2: BlockTensor,
                  R: BlockTensor):
    return ("apply2", theta, L.layout, _mpo_key(W1), _mpo_key(W2), R.layout)


def host_plan_two_site(theta: Layout, L: BlockTensor, W1: BlockTensor, W2: BlockTensor,
                       R: BlockTensor) -> P.HostPlan3:
    """The host tables of the two-site plan (cached; no device copy)."""
    return _real_plan(_two_site_key(theta, L, W1, W2, R),
                      lambda: P.plan_apply(theta, L.layout, [(W1.layout, _host_of(W1)),
                                                             (W2.layout, _host_of(W2))],
                                           R.layout))


def plan_two_site(theta: Layout, L: BlockTensor, W1: BlockTensor, W2: BlockTensor,
                  R: BlockTensor, device, cplx: bool = False, ff: bool = False) -> DevicePlan3:
    key = _two_site_key(theta, L, W1, W2, R)

    def build():
        hp = host_plan_two_site(theta, L, W1, W2, R)
        return DevicePlan3(_cplx(hp) if cplx else hp, device, ff=ff)
    return _PLANS.get_or(key + (str(device), cplx, ff), build)


def plan_one_site(M: Layout, L: BlockTensor, W: BlockTensor, R: BlockTensor,
                  device, cplx: bool = False) -> DevicePlan3:
    key = ("apply1", M, L.layout, _mpo_key(W), R.layout)
    host = lambda: P.plan_apply(M, L.layout, [(W.layout, _host_of(W))], R.layout)
    return _PLANS.get_or(key + (str(device), cplx), lambda: DevicePlan3(
        (_cplx if cplx else (lambda h: h))(_real_plan(key, host)), device))


def plan_left(L: Layout, A: Layout, W: BlockTensor, device, cplx: bool = False,
              ff: bool = False) -> DevicePlan3:
    key = ("left", L, A, _mpo_key(W))
    host = lambda: P.plan_left_env(L, A, (W.layout, _host_of(W)))
    return _PLANS.get_or(key + (str(device), cplx, ff), lambda: DevicePlan3(
        (_cplx if cplx else (lambda h: h))(_real_plan(key, host)), device, ff=ff))


def plan_right(R: Layout, B: Layout, W: BlockTensor, device, cplx: bool = False,
               ff: bool = False) -> DevicePlan3:
    key = ("right", R, B, _mpo_key(W))
    host = lambda: P.plan_right_env(R, B, (W.layout, _host_of(W)))
    return _PLANS.get_or(key + (str(device), cplx, ff), lambda: DevicePlan3(
        (_cplx if cplx else (lambda h: h))(_real_plan(key, host)), device, ff=ff))


def _env_ff(p: DevicePlan3, site: torch.Tensor, env: torch.Tensor, y: torch.Tensor):
    """An environment update in float-float arithmetic: the site tensor and the old environment
    split once into (hi, lo) pairs after the plan's workspace, then tnk_contract3_ff (slots:
    site, env, site)."""
    ns, ne = site.numel(), env.numel()
    need = p.ws_elems
    ws = workspace(need + ns + ne, y.device)
    lib, sp = _lib.lib(), _lib.stream_ptr()
    s2 = ws.data_ptr() + 8 * need
    e2 = s2 + 8 * ns
    _lib.check(lib.tnk_ff_split(site.data_ptr(), s2, ns, sp), "ff split")
    _lib.check(lib.tnk_ff_split(env.data_ptr(), e2, ne, sp), "ff split")
    _lib.check(lib.tnk_contract3_ff(C.byref(p.c), s2, e2, s2, y.data_ptr(), ws.data_ptr(), need,
                                    sp), "tnk_contract3_ff")
    return y


def plan_tdot(a: Layout, b: Layout, nc: int, device, cplx: bool = False) -> DeviceGemmPlan:
    key = ("tdot", a, b, nc)

    def build():
        hp = _real_plan(key, lambda: P.plan_tensordot(a, b, nc))
        if cplx:
            c = P.HostGemmPlan.__new__(P.HostGemmPlan)
            c.g, c.macs, c.out_layout = P.complexify_gemm(hp.g), 4 * hp.macs, hp.out_layout
            hp = c
        return DeviceGemmPlan(hp, device)
    return _PLANS.get_or(key + (str(device), cplx), build)


# --------------------------------------------------------------------------- #
# the reference's hot-path functions on block tensors (tnkit/_dmrg.py:162-231)
# --------------------------------------------------------------------------- #
def _out(p, like, out=None):
    if out is not None:
        return out
    return torch.empty(p.out_layout.size, dtype=like.dtype, device=like.device)


def apply_two_site(theta: BlockTensor, L: BlockTensor, W1: BlockTensor, W2: BlockTensor,
                   R: BlockTensor, out: Optional[torch.Tensor] = None) -> BlockTensor:
    c = _require_cuda(theta.data, L.data, R.data)
    p = plan_two_site(theta.layout, L, W1, W2, R, theta.data.device, c)
    y = _out(p, theta.data, out)
    p.run("tnk_apply_two_site_f64", L.data, theta.data, R.data, y, None)
    return BlockTensor(p.out_layout, y)


def apply_one_site(M: BlockTensor, L: BlockTensor, W: BlockTensor, R: BlockTensor,
                   out: Optional[torch.Tensor] = None) -> BlockTensor:
    c = _require_cuda(M.data, L.data, R.data)
    p = plan_one_site(M.layout, L, W, R, M.data.device, c)
    y = _out(p, M.data, out)
    p.run("tnk_apply_one_site_f64", L.data, M.data, R.data, y, None)
    return BlockTensor(p.out_layout, y)


def update_left_env(L: BlockTensor, A: BlockTensor, W: BlockTensor,
                    precision: str = "f64") -> BlockTensor:
    """L' = A^* L W A (tnkit/_dmrg.py:216-223); precision 'ff' runs it in float-float on real
    tensors (the FP32 CUDA cores, ~1e-14 relative)."""
    c = _require_cuda(L.data, A.data)
    ff = precision == "ff" and not c
    p = plan_left(L.layout, A.layout, W, A.data.device, c, ff=ff)
    y = _out(p, A.data)
    if ff:
        _env_ff(p, A.data, L.data, y)
    else:
        p.run("tnk_update_left_env_f64", A.data, L.data, A.data, y, None)
    return BlockTensor(p.out_layout, y)


def update_right_env(R: BlockTensor, B: BlockTensor, W: BlockTensor,
                     precision: str = "f64") -> BlockTensor:
    """R' = B R W B^* (tnkit/_dmrg.py:224-231); precision 'ff' as in update_left_env."""
    c = _require_cuda(R.data, B.data)
    ff = precision == "ff" and not c
    p = plan_right(R.layout, B.layout, W, B.data.device, c, ff=ff)
    y = _out(p, B.data)
    if ff:
        _env_ff(p, B.data, R.data, y)
    else:
        p.run("tnk_update_right_env_f64", B.data, R.data, B.data, y, None)
    return BlockTensor(p.out_layout, y)


def tensordot(a: BlockTensor, b: BlockTensor, nc: int = 1) -> BlockTensor:
    """Contract the last `nc` legs of a with the first `nc` legs of b (e.g. "asc,ctb->astb")."""
    c = _require_cuda(a.data, b.data)
    p = plan_tdot(a.layout, b.layout, nc, a.data.device, c)
    y = _out(p, a.data)
    p.run(a.data, b.data, y)
    return BlockTensor(p.out_layout, y)


_APPLY2 = {"f64": "tnk_apply_two_site_f64", "ff": "tnk_apply_two_site_ff"}


class TwoSiteOperator:
    """H_eff of one bond as a matvec on flat canonical buffers, for the Krylov solvers: the plan
    and operands are bound once per local problem (tnkit/_dmrg.py:633-675 `matvec`).
    precision 'f64' runs the FP64 grouped GEMM, 'ff' the float-float one (same plan)."""

    def __init__(self, theta_layout: Layout, L: BlockTensor, W1: BlockTensor, W2: BlockTensor,
                 R: BlockTensor, precision: str = "f64", tune: bool = False):
        if precision not in _APPLY2:
            raise ValueError(f"precision must be one of {sorted(_APPLY2)}")
        self.fn = _APPLY2[precision]
        self.precision = precision
        self.cplx = _require_cuda(L.data, R.data)
        self.L, self.R = L, R
        self.device = L.data.device
        ff = precision == "ff"
        self.plan = plan_two_site(theta_layout, L, W1, W2, R, self.device, self.cplx, ff=ff)
        self.n = theta_layout.size
        need = self.plan.ws_elems + (self.plan.out_elems if ff else 0)
        self.ws = workspace(need, self.device)
        if ff:           # float-float copies of the environments, split once per local problem
            lib, sp = _lib.lib(), _lib.stream_ptr()
            self.Lx, self.Rx = torch.empty_like(L.data), torch.empty_like(R.data)
            for src, dst in ((L.data, self.Lx), (R.data, self.Rx)):
                n = src.numel() * (2 if src.is_complex() else 1)
                _lib.check(lib.tnk_ff_split(src.data_ptr(), dst.data_ptr(), n, sp), "ff split")
        else:
            self.Lx, self.Rx = L.data, R.data
        self.calls = 0
        self.inner, self.tuned = None, None
        if tune:
            self._tune(ff)

    def _tune(self, ff: bool):
        """Pick the plan's schedule (inner product, split-K, tile order) by timing the
        candidates on this problem's operands (autotune.tune; cached per shape class)."""
        from . import autotune as AT
        hp = self.plan.host
        dt = torch.complex128 if self.cplx else torch.float64
        xt = torch.randn(self.n, dtype=dt, device=self.device)
        yt = torch.empty_like(xt)

        def run(dp):
            w = workspace(dp.ws_elems + (dp.out_elems if ff else 0), self.device)
            dp.run(self.fn, self.Lx, xt, self.Rx, yt, w)
        t = AT.tune(hp, run, ff=ff)
        self.plan = DevicePlan3(AT.scheduled_plan(hp, t.schedule), self.device, ff=ff)
        self.ws = workspace(self.plan.ws_elems + (self.plan.out_elems if ff else 0),
                            self.device)
        self.inner, self.tuned = t.schedule.inner, t

    @property
    def macs(self):
        return self.plan.macs

    def __call__(self, x: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        y = torch.empty_like(x) if out is None else out
        if self.inner is None:
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


class GraphedOperator:
    """An operator `op(x, out)` replayed from a CUDA graph after one eager warm-up call, as the
    reference's `MatvecGraph` does for its block matvec (tnkit/block_graph.py:124-180): the
    first call runs eagerly (plan uploads, first launches), the second captures the launch
    sequence on static input and output buffers that this wrapper owns, and every call from the
    second on is one graph launch between a copy of the input into the static buffer and a copy
    of the result out of it. The wrapped operator must not allocate, synchronise or read back
    inside its call."""

    def __init__(self, op, n: int, dtype=torch.float64, device=None):
        self.op = op
        self.n = int(n)
        self.dtype = dtype
        self.device = device if device is not None else getattr(op, "device", None)
        self.graph = None
        self.x = self.y = None
        self.eager = 0
        self.replays = 0

    @property
    def calls(self):
        return self.eager + self.replays

    @property
    def macs(self):
        return getattr(self.op, "macs", None)

    def _capture(self):
        self.x = torch.zeros(self.n, dtype=self.dtype, device=self.device)
        self.y = torch.empty(self.n, dtype=self.dtype, device=self.device)
        c0 = getattr(self.op, "calls", 0)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.op(self.x, self.y)
        if hasattr(self.op, "calls"):
            self.op.calls = c0
        self.graph = g

    def __call__(self, x: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        if self.graph is None and self.eager == 0:
            self.eager += 1
            return self.op(x, out)
        if self.graph is None:
            self._capture()
        if x.data_ptr() != self.x.data_ptr():
            self.x.copy_(x.reshape(-1))
        self.graph.replay()
        self.replays += 1
        if out is None:
            return self.y.clone()
        if out.data_ptr() != self.y.data_ptr():
            out.copy_(self.y)
        return out


class OneSiteOperator:
    """H_eff of one site (tnkit/_dmrg.py:192-199) as `op(x, out)` on flat canonical buffers:
    the back-evolution operator of two-site TDVP."""

    def __init__(self, m_layout: Layout, L: BlockTensor, W: BlockTensor, R: BlockTensor):
        self.cplx = _require_cuda(L.data, R.data)
        self.L, self.R = L, R
        self.device = L.data.device
        self.plan = plan_one_site(m_layout, L, W, R, self.device, self.cplx)
        self.ws = workspace(self.plan.ws_elems, self.device)
        self.calls = 0

    def __call__(self, x: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        y = torch.empty_like(x) if out is None else out
        self.plan.run("tnk_apply_one_site_f64", self.L.data, x, self.R.data, y, self.ws)
        self.calls += 1
        return y
