"""`backend="b200"` behind the reference's own front doors.

A process that imports the reference package (tnkit 0.3.0) and this one calls `install()` once;
from then on the reference's unchanged entry points accept the new backend:

    import tnkit
    from tnkit_gb300 import frontdoor
    frontdoor.install()
    Wb, _ = tnkit.to_block_mpo(W, [[1, -1]] * N, tnkit.get_backend("numpy-real"), sym=tnkit.U1())
    E, mps, info = tnkit.dmrg(Wb, 1024, backend="b200", charge=0, expand=0)
    out, records = tnkit.tdvp2_evolve(mps, Wb, 64, 0.05, 20, backend="b200")

What `install` patches (in the reference's modules, nothing on disk):

* `get_backend` (tnkit/backend.py:192-240), in every tnkit module that imported it: the specs
  'b200' (complex128, as 'torch-cuda'), 'b200-real' (float64), 'b200-ff', 'b200-mixed' and
  'b200-mixed-ff' (float64 with the float-float / tensor-core Lanczos) give a `B200Backend`;
  every other spec goes to the reference's own function.
* `_dmrg._dmrg` (tnkit/_dmrg.py:525-799), the sweep that `dmrg` calls by its module-global
  name, so every caller of `dmrg` is covered whatever it imported: when the options name a b200
  backend (a spec above, a `B200Backend`, or `BlockBackend(B200Backend(...))`), the whole sweep
  -- the reference's `solve_block` (:677-727) with its matvec, Lanczos, truncation and
  environment updates -- runs in this package (`tnkit_gb300.dmrg.dmrg`) on the GPU, the
  reference's block MPO and initial state converted in with `BlockTensor.from_reference`
  (the reference's own canonical buffer, copied to the device as it is). The state comes back
  as the reference's `BlockTensor`s (dense MPOs: dense tensors) with CUDA torch buffers, as
  `tnkit.mps.MPS(..., center=0)`, and `info` carries the reference's keys.
* `tdvp._tdvp2` (tnkit/tdvp.py:704-800): the same for two-site TDVP; the reference's
  `_evolve_two_site` (:555-650) per bond becomes `tnkit_gb300.tdvp.tdvp2_evolve`'s. `measure`
  sees the state as the reference's tensors.

Options the GPU path does not implement raise `NotImplementedError` when they differ from the
reference's defaults (never silently ignored). Subspace expansion is one of them: the reference
expands block DMRG by default (`expand=None` means up to 4 expansion sweeps), so with b200 pass
`expand=0`. `uninstall()` puts the reference's functions back.
"""
from __future__ import annotations

import dataclasses
import sys
from typing import Any, Dict, Optional

import numpy as np

_STATE: Dict[str, Any] = {}

_PRECISIONS = {"b200": "f64", "b200-real": "f64", "b200-ff": "ff", "b200-mixed": "mixed",
               "b200-mixed-ff": "mixed-ff"}


def b200_precision(backend) -> Optional[str]:
    """The precision a backend spec asks of this package, or None when it names another
    backend: a spec string of `_PRECISIONS`, a `B200Backend`, or a block adaptor around one."""
    from .backend import B200Backend
    if isinstance(backend, str):
        return _PRECISIONS.get(backend)
    if isinstance(backend, B200Backend):
        return backend.precision
    dense = vars(backend).get("dense") if hasattr(backend, "__dict__") else None
    if isinstance(dense, B200Backend):
        return dense.precision
    return None


def _ref_get_backend(spec, **kw):
    from .backend import B200Backend
    if isinstance(spec, str) and spec in _PRECISIONS:
        return B200Backend.from_spec(spec)
    return _STATE["get_backend"](spec, **kw)


def _patch_everywhere(original, replacement):
    for name, mod in list(sys.modules.items()):
        if mod is None or not (name == "tnkit" or name.startswith("tnkit.")):
            continue
        for attr in ("get_backend",):
            if getattr(mod, attr, None) is original:
                setattr(mod, attr, replacement)


def install(tnkit=None):
    """Register backend 'b200' with the imported reference package (idempotent). Returns it."""
    if tnkit is None:
        import tnkit
    if _STATE.get("installed"):
        return tnkit
    from tnkit import _dmrg as rd
    from tnkit import backend as rb
    from tnkit import tdvp as rt
    _STATE.update(tnkit=tnkit, get_backend=rb.get_backend, dmrg_core=rd._dmrg,
                  tdvp2_core=rt._tdvp2)
    _patch_everywhere(rb.get_backend, _ref_get_backend)

    def _dmrg(mpo, chi, o):
        prec = b200_precision(o.backend)
        if prec is None:
            return _STATE["dmrg_core"](mpo, chi, o)
        return run_dmrg(mpo, chi, o, prec)

    def _tdvp2(mps, mpo, chi, dt, n_steps, o):
        prec = b200_precision(o.backend)
        if prec is None:
            return _STATE["tdvp2_core"](mps, mpo, chi, dt, n_steps, o)
        return run_tdvp2(mps, mpo, chi, dt, n_steps, o, prec)

    rd._dmrg = _dmrg
    rt._tdvp2 = _tdvp2
    _STATE["installed"] = True
    return tnkit


def uninstall():
    """Put the reference's own functions back."""
    if not _STATE.get("installed"):
        return
    from tnkit import _dmrg as rd
    from tnkit import tdvp as rt
    _patch_everywhere(_ref_get_backend, _STATE["get_backend"])
    rd._dmrg = _STATE["dmrg_core"]
    rt._tdvp2 = _STATE["tdvp2_core"]
    _STATE.clear()


# --- conversions between the reference's tensors and this package's --------------------------

def _device():
    """The CUDA device the sweeps run on: the current one."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("backend 'b200' needs a CUDA device (GB300)")
    return torch.device("cuda", torch.cuda.current_device())


def _is_block(x) -> bool:
    return bool(getattr(x, "is_block", False)) and hasattr(x, "struct")


def from_reference_tensor(t, device, dtype=None):
    """This package's BlockTensor of a reference BlockTensor (its canonical buffer, moved to the
    device as it is)."""
    from .tensor import BlockTensor
    return BlockTensor.from_reference(t, device=device, dtype=dtype)


def to_reference_tensor(t, sym, tnkit=None):
    """The reference's BlockTensor with this tensor's legs, charge and device buffer (no copy):
    the canonical layouts are the same, block for block."""
    tnkit = tnkit or _STATE.get("tnkit") or __import__("tnkit")
    from tnkit import blocks as RB
    legs = tuple(RB.Leg(tuple(l.charges), tuple(int(d) for d in l.dims), int(l.sign), sym)
                 for l in t.layout.legs)
    st = RB.canonical(legs, sym.label(t.layout.charge))
    if st.size != t.layout.size:
        raise RuntimeError("the reference's canonical layout differs from this package's")
    return RB.BlockTensor(st, t.data.contiguous())


def _dense_in(W) -> np.ndarray:
    if hasattr(W, "detach"):
        W = W.detach().cpu().numpy()
    return np.asarray(W)


def _dense_mps_in(mps, device, dtype=None):
    """Dense (left, phys, right) site tensors as this package's one-block tensors."""
    import torch
    from .layout import Leg, layout_of
    from .tensor import BlockTensor
    out = []
    for A in mps:
        a = torch.as_tensor(A.detach() if hasattr(A, "detach") else np.asarray(A))
        if dtype is None and not torch.is_complex(a):
            a = a.to(torch.float64)
        a = a.to(device=device, dtype=dtype or a.dtype).contiguous()
        l, d, r = (int(x) for x in a.shape)
        lay = layout_of((Leg((0,), (l,), 1), Leg((0,), (d,), 1), Leg((0,), (r,), -1)), 0)
        out.append(BlockTensor(lay, a.reshape(-1)))
    return out


def _dense_mps_out(M):
    """One-block site tensors back as dense (left, phys, right) device tensors (views)."""
    return [m.data.view(*(int(l.size) for l in m.layout.legs)) for m in M]


def _check_options(o, supported, what):
    """Refuse every option field outside `supported` that differs from the reference default."""
    default = type(o)()
    for f in dataclasses.fields(o):
        if f.name in supported:
            continue
        v, d = getattr(o, f.name), getattr(default, f.name)
        same = v is d or (type(v) is type(d) and _equal(v, d))
        if not same:
            raise NotImplementedError(f"{what} with backend 'b200' does not take "
                                      f"{f.name}={v!r} (the GPU path implements the reference's "
                                      f"default, {d!r})")


def _equal(a, b) -> bool:
    try:
        return bool(a == b)
    except Exception:
        return False


_DMRG_TAKES = {"n_sweeps", "tol", "rtol", "trunc", "eig_tol", "eig", "warm_start", "seed",
               "init_mps", "backend", "max_iter", "verbose", "restart_m", "restart_k",
               "mixed_tol_lo", "charge", "sites", "expand", "expand_alpha", "expand_decay"}


def run_dmrg(mpo, chi, o, precision: str = "f64"):
    """The reference's `_dmrg(mpo, chi, o)` on this package's GPU sweep."""
    import torch
    from .dmrg import dmrg
    tnkit = _STATE.get("tnkit") or __import__("tnkit")
    _check_options(o, _DMRG_TAKES, "dmrg")
    if o.sites != 2:
        raise NotImplementedError("backend 'b200' runs two-site DMRG (sites=2)")
    if o.trunc not in ("svd", "gram"):
        raise NotImplementedError(f"backend 'b200' truncates with trunc='svd' or 'gram', "
                                  f"not {o.trunc!r}")
    block = _is_block(mpo[0])
    expand = o.expand
    if expand is None:       # the reference's default (tnkit/_dmrg.py:562-563)
        expand = min(4, max(0, o.n_sweeps - 2)) if block else 0
    if expand:
        raise NotImplementedError("subspace expansion is not part of backend 'b200'; pass "
                                  "expand=0 (the reference's block default expands)")
    eig = o.eig
    if eig == "lanczos-mixed":
        precision = "mixed" if precision == "f64" else precision
        eig = "lanczos-restart"
    if eig != "lanczos-restart":
        raise NotImplementedError(f"backend 'b200' solves with eig='lanczos-restart' or "
                                  f"'lanczos-mixed', not {eig!r}")
    device = _device()
    if block:
        sym = mpo[0].struct.sym
        W = [from_reference_tensor(w, device) for w in mpo]
        init = None if o.init_mps is None else \
            [from_reference_tensor(m, device) for m in o.init_mps]
    else:
        sym = None
        W = [_dense_in(w) for w in mpo]
        init = None if o.init_mps is None else _dense_mps_in(o.init_mps, device)
    E, M, info = dmrg(W, chi, n_sweeps=o.n_sweeps, tol=o.tol, rtol=o.rtol, eig_tol=o.eig_tol,
                      warm_start=o.warm_start, seed=o.seed, init_mps=init,
                      max_iter=o.max_iter, verbose=o.verbose, restart_m=o.restart_m,
                      restart_k=o.restart_k, mixed_tol_lo=o.mixed_tol_lo, charge=o.charge,
                      expand=0, precision=precision,
                      svd_method="gram" if o.trunc == "gram" else "svd")
    out = [to_reference_tensor(m, sym, tnkit) for m in M] if block else \
        _dense_mps_out(M)
    info = dict(info)
    info["backend"] = "b200"
    info["eig"] = o.eig
    return E, tnkit.mps.MPS(out, center=0), info


_TDVP_TAKES = {"backend", "measure", "meas_every", "trunc", "chi_max", "renorm", "seed",
               "canonicalize", "keep_device", "krylov_m", "profile", "fast_expm"}


def run_tdvp2(mps, mpo, chi, dt, n_steps, o, precision: str = "f64"):
    """The reference's `_tdvp2(mps, mpo, chi, dt, n_steps, o)` on this package's GPU sweep."""
    import torch
    from .mpo import dense_mpo
    from .tdvp import tdvp2_evolve
    tnkit = _STATE.get("tnkit") or __import__("tnkit")
    if callable(mpo):
        raise NotImplementedError("backend 'b200' evolves under a time-independent MPO")
    _check_options(o, _TDVP_TAKES, "tdvp2_evolve")
    if o.trunc not in ("svd", "gram"):
        raise NotImplementedError(f"backend 'b200' truncates with trunc='svd' or 'gram', "
                                  f"not {o.trunc!r}")
    if precision != "f64":
        raise NotImplementedError("backend 'b200' evolves in complex128 (FP64)")
    device = _device()
    block = _is_block(mps[0])
    if block != _is_block(mpo[0]):
        raise ValueError("block tensors need a block MPS and a block MPO")
    if block:
        sym = mpo[0].struct.sym
        W = [from_reference_tensor(w, device) for w in mpo]
        M = [from_reference_tensor(m, device, dtype=torch.complex128) for m in mps]
        back = lambda ms: [to_reference_tensor(m, sym, tnkit) for m in ms]
    else:
        W = dense_mpo([_dense_in(w) for w in mpo], device=device)
        M = _dense_mps_in(mps, device, dtype=torch.complex128)
        back = _dense_mps_out
    measure = None if o.measure is None else (lambda ms: o.measure(back(ms)))
    cap = int(chi if o.chi_max is None else o.chi_max)
    fe = o.fast_expm
    if isinstance(fe, dict):            # the reference's re-entrant form: its fixed m, or 'auto'
        fe = fe.get("m") or "auto"
    prof = {} if o.profile is not None else None
    out, records = tdvp2_evolve(M, W, cap, dt, n_steps, measure=measure,
                                meas_every=o.meas_every, krylov_m=o.krylov_m, renorm=o.renorm,
                                canonicalize=o.canonicalize, profile=prof,
                                svd_method="gram" if o.trunc == "gram" else "svd",
                                fast_expm=fe)
    if prof is not None:
        o.profile.update(prof)
    centre = 0 if (o.canonicalize or n_steps > 0) else None
    return tnkit.mps.MPS(back(out), center=centre), records
