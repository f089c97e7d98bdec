"""Krylov (Lanczos) exponential exp(tau H) v on the GPU for complex128 vectors
(tnkit/eigensolver.py:230-349 `lanczos_expm` with its `_ExpmMonitor`; block twin
tnkit/block_lanczos.py:76-121).

The Krylov basis stays on the device; each step is one matvec, the three-term subtraction, two
classical Gram-Schmidt passes against the whole basis (tnk_zmultidot_f64 + tnk_zgemv_sub_f64:
the full reorthogonalisation of the reference, as two batched passes), and the norm. The host
reads the step's alpha and beta in one small copy and runs the reference's monitor: stop on
breakdown (beta < tol) or when Saad's a-posteriori estimate of the first neglected term,
|beta| |tau| |exp(tau T)[j-1, 0]| ||v||, falls below tol (from j >= 2); the coefficients are
||v|| exp(tau T) e_1 of the projected tridiagonal T.
"""
from __future__ import annotations

import math
from typing import Callable, Optional

import numpy as np
import scipy.linalg
import torch

from . import _lib

_MAXNV = 64


def _expm_col(tau, alphas, betas, route: str = "eigh") -> np.ndarray:
    """The first column of exp(tau T) for the real symmetric tridiagonal T of the Lanczos
    coefficients. 'eigh' (default): T = Z diag(lam) Z^T by LAPACK's tridiagonal solver, then
    exp(tau T) e_1 = Z (exp(tau lam) * Z[0, :]) -- exact to eigensolver accuracy, O(j^2) after
    the O(j^2) eigensolve, the route the reference offers as `expm_sym_tridiag_eigh`
    (tnkit/backend.py:643-661); 'pade': scipy's scaling and squaring on the complex j x j
    matrix, the reference's per-iteration host call (tnkit/eigensolver.py:260)."""
    j = len(alphas)
    if route == "pade":
        return scipy.linalg.expm(tau * _tridiag(alphas, betas))[:, 0]
    if route != "eigh":
        raise ValueError("route must be 'eigh' or 'pade'")
    d = np.asarray(alphas, np.float64)
    if j == 1:
        return np.exp(tau * d).astype(complex)
    lam, Z = scipy.linalg.eigh_tridiagonal(d, np.asarray(betas[:j - 1], np.float64),
                                           check_finite=False)
    return Z @ (np.exp(tau * lam) * Z[0, :])


def _tridiag(alphas, betas) -> np.ndarray:
    j = len(alphas)
    T = np.diag(np.asarray(alphas, np.float64)).astype(complex)
    if j > 1:
        off = np.asarray(betas[:j - 1], np.float64)
        T += np.diag(off, 1) + np.diag(off, -1)
    return T


class ExpmMonitor:
    """Breakdown test, Saad's estimate, adaptive stop and the final coefficients."""

    def __init__(self, tau, beta0, tol, adaptive, info, est_ref_j=2, route="eigh"):
        self.tau, self.beta0, self.tol, self.adaptive = tau, beta0, tol, adaptive
        self.route = route
        self.info, self.est_ref_j = info, est_ref_j
        self.est = float("inf")
        self.est_ref, self.est_ref_at, self.beta1 = float("nan"), 0, float("nan")

    def check(self, k, alphas, betas, beta):
        if k == 0:
            self.beta1 = beta
        if beta < self.tol:
            if self.info is not None and self.est_ref_at == 0:
                self.est_ref, self.est_ref_at = 0.0, k + 1
            return "breakdown"
        jj = len(alphas)
        want_ref = self.info is not None and self.est_ref_at == 0 and jj >= self.est_ref_j
        if (self.adaptive and jj >= 2) or want_ref:
            e1 = _expm_col(self.tau, alphas, betas, self.route)
            self.est = abs(beta) * abs(self.tau) * abs(e1[jj - 1]) * self.beta0
            if want_ref:
                self.est_ref, self.est_ref_at = self.est, jj
            if self.adaptive and jj >= 2 and self.est < self.tol:
                return "converged"
        return None

    def finish(self, alphas, betas, capped):
        c = self.beta0 * _expm_col(self.tau, alphas, betas, self.route)
        if self.info is not None:
            self.info.update(krylov_dim=len(alphas), err_est=self.est, beta1=self.beta1,
                             est_ref=self.est_ref, est_ref_j=self.est_ref_at, capped=capped)
        return c


def _real(x: torch.Tensor) -> torch.Tensor:
    return torch.view_as_real(x).reshape(-1)


def lanczos_expm(matvec: Callable, v: torch.Tensor, tau: complex, m: int = 30,
                 tol: float = 1e-12, adaptive: bool = True, info: Optional[dict] = None,
                 est_ref_j: int = 2, route: str = "eigh") -> torch.Tensor:
    """exp(tau H) v for Hermitian H given as `matvec(x, out)` on complex128 CUDA vectors. The
    per-iteration Saad estimate and the final coefficients take exp(tau T) e_1 by `route`
    ('eigh': the tridiagonal eigendecomposition; 'pade': scipy's expm of the j x j matrix)."""
    if not (v.is_cuda and v.dtype == torch.complex128):
        raise TypeError("lanczos_expm needs a complex128 CUDA vector")
    if m + 1 > _MAXNV:
        raise ValueError(f"Krylov dimension {m} exceeds {_MAXNV - 1}")
    lib = _lib.lib()
    sp = _lib.stream_ptr()
    dev = v.device
    v = v.reshape(-1)
    n = v.numel()
    red = torch.empty(_lib.TNK_RED_ELEMS, dtype=torch.float64, device=dev)
    # slots: [0] beta0, [1] beta, [8 : 8+2*64] pass-1 coefficients, then pass-2 coefficients
    sc = torch.zeros(8 + 4 * _MAXNV, dtype=torch.float64, device=dev)
    host = torch.zeros(8 + 4 * _MAXNV, dtype=torch.float64, pin_memory=True)
    a = lambda i: sc.data_ptr() + 8 * i
    c1, c2 = 8, 8 + 2 * _MAXNV

    def read():
        host.copy_(sc, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return host

    _lib.check(lib.tnk_nrm2_f64(_real(v).data_ptr(), 2 * n, a(0), red.data_ptr(), sp), "nrm2")
    beta0 = float(read()[0])
    if not math.isfinite(beta0) or beta0 < 1e-300:
        return v.clone()
    mon = ExpmMonitor(tau, beta0, tol, adaptive, info, est_ref_j, route)
    V = torch.empty((m + 1, n), dtype=torch.complex128, device=dev)
    _lib.check(lib.tnk_scale_div_f64(_real(v).data_ptr(), _real(V[0]).data_ptr(), 2 * n, a(0),
                                     1.0, sp), "scale_div")
    w = torch.empty(n, dtype=torch.complex128, device=dev)
    alphas, betas = [], []
    beta = 0.0
    capped = False
    nv = 1
    for k in range(m):
        matvec(V[k], w)
        if k > 0:
            _lib.check(lib.tnk_zaxpby_f64(V[k - 1].data_ptr(), w.data_ptr(), n, None, -beta,
                                          None, 1.0, sp), "zaxpby")
        nv = k + 1
        for slot in (c1, c2):
            _lib.check(lib.tnk_zmultidot_f64(V.data_ptr(), n, nv, w.data_ptr(), n, a(slot),
                                             red.data_ptr(), sp), "zmultidot")
            _lib.check(lib.tnk_zgemv_sub_f64(V.data_ptr(), n, nv, a(slot), w.data_ptr(), n, sp),
                       "zgemv_sub")
        _lib.check(lib.tnk_nrm2_f64(_real(w).data_ptr(), 2 * n, a(1), red.data_ptr(), sp),
                   "nrm2")
        h = read()
        alpha = float(h[c1 + 2 * k])          # Re <V_k, w> after the three-term subtraction
        beta = float(h[1])
        alphas.append(alpha)
        stop = mon.check(k, alphas, betas, beta)
        if stop == "breakdown":
            break
        betas.append(beta)
        _lib.check(lib.tnk_scale_div_f64(_real(w).data_ptr(), _real(V[k + 1]).data_ptr(), 2 * n,
                                         a(1), 1.0, sp), "scale_div")
        if stop:
            break
    else:
        capped = bool(adaptive)
    coef = mon.finish(alphas, betas, capped)
    out = torch.zeros(n, dtype=torch.complex128, device=dev)
    cneg = torch.as_tensor(np.stack([-coef.real, -coef.imag], -1).reshape(-1),
                           dtype=torch.float64, device=dev)
    _lib.check(lib.tnk_zgemv_sub_f64(V.data_ptr(), n, len(coef), cneg.data_ptr(),
                                     out.data_ptr(), n, sp), "zgemv_sub")
    torch.cuda.current_stream().synchronize()
    return out
