"""Two-site DMRG on the GPU with the reference's front door (tnkit/_dmrg.py:312-522).

`dmrg(mpo, chi, options=None, **kw) -> (E, mps, info)` runs the reference's sweep
(tnkit/_dmrg.py:560-799) for block (U(1)) and dense MPOs: a seeded random start drawn as the
reference draws it, right canonicalisation by per-block LQ, right environments, then sweeps of
`solve_block` -- theta = M_i M_i+1, thick-restart Lanczos on H_eff, truncated SVD across sectors,
environment growth. Every contraction of the loop runs in the tnk_* kernels; the Krylov vectors,
environments and MPS tensors stay on the device.

Options keep the reference's names and defaults where this backend implements them
(`n_sweeps`, `tol`, `rtol`, `eig_tol`, `eig`, `warm_start`, `max_iter`, `restart_m`, `restart_k`,
`seed`, `init_mps`, `charge`, `verbose`, `sites`, `expand`, `trunc`, `backend`, `precision`;
`mixed_schedule='sweep'` solves the opening sweeps on the tensor cores alone and polishes only
the last `polish_sweeps`). The
block default of the reference expands the subspace in the opening sweeps; subspace expansion is
not part of this backend, so `expand` must be 0 (or None, read as 0) and other values raise.
"""
from __future__ import annotations

import dataclasses
import time
from typing import Any, List, Optional

import numpy as np
import torch

from . import linalg as LA
from . import ops
from .lanczos import lanczos_ground_restart
from .layout import canonical
from .mpo import dense_mpo, random_block_mps, random_dense_mps
from .tensor import BlockTensor


@dataclasses.dataclass
class DMRGOptions:
    n_sweeps: int = 8
    tol: float = 1e-10
    trunc: str = "svd"
    eig_tol: float = 1e-9
    eig: str = "lanczos-restart"
    warm_start: bool = True
    seed: int = 0
    init_mps: Optional[List[BlockTensor]] = None
    backend: Any = "b200"
    max_iter: Optional[int] = None
    verbose: bool = False
    restart_m: int = 40
    restart_k: int = 10
    charge: Any = None
    sites: int = 2
    expand: Optional[int] = None
    rtol: float = 1e-10
    precision: str = "f64"          # 'f64', 'ff' (float-float), 'mixed' or 'mixed-ff'
                                    # (tensor-core Lanczos, then an FP64 / float-float polish)
    mixed_tol_lo: float = 1e-4
    polish: int = 2                  # FP64 polish restarts allowed after the mixed stage
    mixed_schedule: str = "bond"     # 'bond': tensor-core stage then polish at every bond;
                                     # 'sweep': tensor-core solves alone in all but the last
                                     # `polish_sweeps` sweeps, the per-bond mixed solve there
    polish_sweeps: int = 2
    polish_mode: str = "lanczos"          # mixed modes: 'lanczos' (high-precision Lanczos from the
                                          # tensor-core vector) or 'refine' (defect correction:
                                          # high-precision residuals, tensor-core correction
                                          # solves, Lanczos only if still above eig_tol)
    device: Any = None
    svd_driver: Optional[str] = "gesvd"   # cuSOLVER driver of the per-sector SVD (as the reference)
    svd_method: str = "svd"               # 'svd' (exact) or 'gram' (eigh of the Gram matrix)
    svd_host: str = "auto"                # with 'gram': where the sectors factor ('device':
                                          # reduction and back-transformation on the GPU, the
                                          # tridiagonal eigenproblems on the host; 'never': per
                                          # sector on cuSOLVER; 'always': host LAPACK; 'auto':
                                          # the default route of truncated_svd)
    env_precision: str = "auto"           # 'f64', 'ff' (environment updates in float-float:
                                          # ~2x faster, ~10x larger energy error, ~1e-13) or
                                          # 'auto': float-float in the tensor-core-only sweeps
                                          # of the 'sweep' schedule, FP64 everywhere else
    graph: bool = False                   # replay each local problem's FP64 / float-float
                                          # matvec from a CUDA graph after one eager call
                                          # (as the reference's MatvecGraph)


def _resolve(options, kw) -> DMRGOptions:
    if options is None:
        o = DMRGOptions()
    elif isinstance(options, dict):
        o = DMRGOptions(**options)
    else:
        o = dataclasses.replace(options)
    names = {f.name for f in dataclasses.fields(DMRGOptions)}
    for k, v in kw.items():
        if k not in names:
            raise TypeError(f"dmrg() got an unexpected keyword argument {k!r}")
        setattr(o, k, v)
    return o


def edge_envs(M: List[BlockTensor], mpo: List[BlockTensor], device):
    """Trivial boundary environments with the legs of the outer bonds and MPO channels
    (tnkit/_dmrg.py:234-247)."""
    a, b = M[0].legs[0], M[-1].legs[2]
    lay_l = canonical((a, mpo[0].legs[0].flip(), a.flip()), 0)
    lay_r = canonical((b, mpo[-1].legs[1].flip(), b.flip()), 0)
    one = lambda lay: BlockTensor(lay, torch.ones(lay.size, dtype=torch.float64, device=device))
    if lay_l.size != 1 or lay_r.size != 1:
        raise ValueError("open boundaries need one-dimensional outer bonds and MPO channels")
    return one(lay_l), one(lay_r)


def right_canonicalize(M: List[BlockTensor], scal: LA.Scalars) -> List[BlockTensor]:
    """Right-canonical form by per-block LQ from the right, centre renormalised at every step
    (tnkit/_dmrg.py:295-306)."""
    for i in range(len(M) - 1, 0, -1):
        f, info = LA.fuse_matrix(M[i], 1)
        Lm, Q = LA.lq(f)
        M[i] = LA.split_cols(Q, info)
        Lm = LA.split_rows(Lm, info)
        M[i - 1] = ops.tensordot(M[i - 1], Lm, 1)
        scal.normalize_(M[i - 1].data)
    scal.normalize_(M[0].data)
    return M


def setup_chain(mpo, chi: int, o: DMRGOptions, device):
    """MPO tensors on the device, the initial MPS (o.init_mps, or the seeded random one),
    right-canonicalised, and the environments of a sweep's start: (W, M, L, R, block)."""
    block = isinstance(mpo[0], BlockTensor)
    if block and (o.charge is None) == (o.init_mps is None):
        raise ValueError("a block MPO needs exactly one of charge= and a block init_mps")
    if not block and o.charge is not None:
        raise ValueError("charge= needs a block MPO (convert it with to_block_mpo first)")
    N = len(mpo)
    if block:
        W = list(mpo)
        for w in W:
            if w.data.device != device:
                w.data = w.data.to(device)
    else:
        W = dense_mpo([np.asarray(w) for w in mpo], device=device)
    if o.init_mps is not None:
        M = [BlockTensor(m.layout, m.data.to(device).clone()) for m in o.init_mps]
    elif block:
        M = random_block_mps(W, chi, o.charge, np.random.default_rng(o.seed), device=device)
    else:
        d = W[0].legs[2].size
        M = random_dense_mps(N, chi, d, np.random.default_rng(o.seed), device=device)
    M = right_canonicalize(M, LA.Scalars(device))
    L: List[Optional[BlockTensor]] = [None] * (N + 1)
    R: List[Optional[BlockTensor]] = [None] * (N + 1)
    L[0], R[N] = edge_envs(M, W, device)
    for i in range(N - 1, 0, -1):
        R[i] = ops.update_right_env(R[i + 1], M[i], W[i])
    return W, M, L, R, block


def dmrg(mpo, chi: Optional[int] = None, options=None, **kw):
    """Ground state of an MPO by two-site DMRG on the GPU. See the module docstring."""
    if chi is None:
        chi = kw.pop("chi", None)
        if chi is None:
            raise TypeError("dmrg() missing required argument 'chi' (bond dimension)")
    o = _resolve(options, kw)
    if o.precision not in ("f64", "ff", "mixed", "mixed-ff"):
        raise ValueError("precision must be 'f64', 'ff', 'mixed' or 'mixed-ff'")
    if o.mixed_schedule not in ("bond", "sweep"):
        raise ValueError("mixed_schedule must be 'bond' or 'sweep'")
    if o.sites != 2:
        raise NotImplementedError("this backend runs two-site DMRG (sites=2)")
    if o.trunc != "svd":
        raise ValueError("this backend truncates with trunc='svd'")
    if o.eig not in ("lanczos-restart", "lanczos-mixed"):
        raise ValueError("this backend's local solver is 'lanczos-restart' ('lanczos-mixed' with "
                         "precision='mixed')")
    expand = 0 if o.expand is None else o.expand
    if expand != 0:
        raise NotImplementedError("subspace expansion is not part of this backend: pass expand=0")
    if o.n_sweeps < 1:
        raise ValueError("n_sweeps must be >= 1")
    device = torch.device(o.device) if o.device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    W, M, L, R, block = setup_chain(mpo, chi, o, device)
    N = len(W)

    if o.env_precision not in ("f64", "ff", "auto"):
        raise ValueError("env_precision must be 'f64', 'ff' or 'auto'")

    def env_prec():
        if o.env_precision == "auto":
            return "ff" if tc_only_sweep() else "f64"
        return o.env_precision
    energies, sweep_s, alphas, disc_sweeps = [], [], [], []
    phase = {"eig": 0.0, "trunc": 0.0, "env": 0.0}
    counts = {"lo": 0, "hi": 0}
    total_disc, mv_calls = 0.0, 0
    basis = {"buf": None}

    def sync():
        torch.cuda.current_stream().synchronize()

    def tc_only_sweep():
        return (o.precision in ("mixed", "mixed-ff") and o.mixed_schedule == "sweep"
                and sweep_no["n"] < o.n_sweeps - max(0, o.polish_sweeps))

    def eigsolve(theta: BlockTensor, i: int):
        nonlocal mv_calls
        hi = "ff" if o.precision in ("ff", "mixed-ff") else "f64"
        tc_only = tc_only_sweep()
        op = None if tc_only else ops.TwoSiteOperator(theta.layout, L[i], W[i], W[i + 1],
                                                      R[i + 2], precision=hi)
        if o.graph and op is not None:
            op = ops.GraphedOperator(op, theta.layout.size, device=device)
        n = theta.layout.size
        mi = o.max_iter if o.max_iter is not None else min(n, max(200, 4 * chi))
        need = (o.restart_m + 1) * n
        if basis["buf"] is None or basis["buf"].numel() < need:
            basis["buf"] = torch.empty(need, dtype=torch.float64, device=device)
        Vb = basis["buf"][:need].view(o.restart_m + 1, n)
        v0 = theta.data if o.warm_start else torch.as_tensor(
            np.random.default_rng(o.seed + 1).standard_normal(n), device=device)
        if o.precision in ("mixed", "mixed-ff"):
            from .mixed import mixed_ground
            e, x, info = mixed_ground(theta.layout, L[i], W[i], W[i + 1], R[i + 2], op, v0,
                                      tol=o.eig_tol, max_iter=mi, m=o.restart_m,
                                      k=o.restart_k, tol_lo=o.mixed_tol_lo, basis=Vb,
                                      counts=counts, tc_only=tc_only,
                                      polish_mode=o.polish_mode)
        else:
            e, x, info = lanczos_ground_restart(op, v0, tol=o.eig_tol, max_iter=mi,
                                                m=o.restart_m, k=o.restart_k, basis=Vb)
            counts["hi"] += op.calls
        mv_calls += info["matvecs"] if "matvecs" in info else op.calls
        return e, BlockTensor(theta.layout, x)

    def solve_block(i: int, right: bool):
        nonlocal total_disc
        t0 = time.perf_counter()
        theta0 = ops.tensordot(M[i], M[i + 1], 1)
        e, x = eigsolve(theta0, i)
        sync()
        phase["eig"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        mat, info = LA.fuse_matrix(x, 2)
        U, S, Vh, disc = LA.truncated_svd(mat, chi, scale="right" if right else "left",
                                          driver=o.svd_driver, method=o.svd_method,
                                          host=o.svd_host)
        M[i] = LA.split_rows(U, info)
        M[i + 1] = LA.split_cols(Vh, info)
        total_disc += disc
        sync()
        phase["trunc"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        if right:
            L[i + 1] = ops.update_left_env(L[i], M[i], W[i], precision=env_prec())
        else:
            R[i + 1] = ops.update_right_env(R[i + 2], M[i + 1], W[i + 1],
                                            precision=env_prec())
        sync()
        phase["env"] += time.perf_counter() - t0
        return e

    prev_E, E = None, None
    sweep = 0
    sweep_no = {"n": 0}
    for sweep in range(o.n_sweeps):
        sweep_no["n"] = sweep
        sync()
        ts = time.perf_counter()
        alphas.append(0.0)
        for i in range(0, N - 1):
            E = solve_block(i, True)
        for i in range(N - 2, -1, -1):
            E = solve_block(i, False)
        energies.append(E)
        disc_sweeps.append(total_disc - sum(disc_sweeps))
        sync()
        sweep_s.append(time.perf_counter() - ts)
        if o.verbose:
            print(f"  sweep {sweep + 1:2d}: E = {E:.12f}  (chi={chi}, b200, {o.precision})",
                  flush=True)
        if prev_E is not None and abs(E - prev_E) < max(o.tol, o.rtol * abs(E)):
            break
        prev_E = E
    info = {"sweeps": sweep + 1, "energies": energies, "backend": "b200", "blocks": block,
            "eig": o.eig, "discarded_weight": total_disc, "discarded_per_sweep": disc_sweeps,
            "matvec_calls": mv_calls,
            "phase_time": phase, "mixed_counts": counts, "sites": 2, "expand": 0,
            "expand_alphas": alphas, "sweep_s": sweep_s, "precision": o.precision}
    return E, M, info
