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


def lanczos_expm_fixed(matvec: Callable, v: torch.Tensor, tau: complex, m: int,
                       info: Optional[dict] = None) -> torch.Tensor:
    """exp(tau H) v from exactly `m` Lanczos steps with no host round trip (the reference's
    lanczos_expm_fixed, tnkit/eigensolver.py:95-217, with its 'eigh' route): every Lanczos
    coefficient stays in device memory -- the three-term subtraction, the two CGS passes and
    the normalisation read alpha and beta from there -- and the tridiagonal's eigendecomposition
    (tnk_tridiag_eig_f64), the coefficients beta0 exp(tau T) e_1 and the combination of the
    basis run on the device after the last step. Breakdown needs no branch: a beta at
    rounding level is clamped (the reference's guard_denom) before it divides, and the
    coefficients of the later vectors are at rounding level. Nothing is read back; the caller
    synchronises when it needs the result. `m` is capped at the vector length."""
    if not (v.is_cuda and v.dtype == torch.complex128):
        raise TypeError("lanczos_expm_fixed needs a complex128 CUDA vector")
    from .tridiag import tridiag_eigh_batched
    lib = _lib.lib()
    sp = _lib.stream_ptr()
    dev = v.device
    v = v.reshape(-1)
    n = v.numel()
    m = max(1, min(int(m), n))
    if m + 1 > _MAXNV:
        raise ValueError(f"Krylov dimension {m} exceeds {_MAXNV - 1}")
    red = torch.empty(_lib.TNK_RED_ELEMS, dtype=torch.float64, device=dev)
    c1 = torch.zeros(2 * _MAXNV, dtype=torch.float64, device=dev)
    c2 = torch.zeros(2 * _MAXNV, dtype=torch.float64, device=dev)
    # beta_k as complex numbers (beta, 0) in bc[2k], bc[2k+1]; beta0 in b0[0], b0[1] = 0
    bc = torch.zeros(2 * (m + 1), dtype=torch.float64, device=dev)
    b0 = torch.zeros(2, dtype=torch.float64, device=dev)
    alph = torch.zeros(m, dtype=torch.float64, device=dev)
    V = torch.empty((m, n), dtype=torch.complex128, device=dev)
    w = torch.empty(n, dtype=torch.complex128, device=dev)
    _lib.check(lib.tnk_nrm2_f64(_real(v).data_ptr(), 2 * n, b0.data_ptr(), red.data_ptr(), sp),
               "nrm2")
    beta0 = b0[:1].clone()
    b0[:1].clamp_(min=1e-200)
    _lib.check(lib.tnk_scale_div_f64(_real(v).data_ptr(), _real(V[0]).data_ptr(), 2 * n,
                                     b0.data_ptr(), 1.0, sp), "scale_div")
    for k in range(m):
        matvec(V[k], w)
        if k > 0:
            _lib.check(lib.tnk_zaxpby_f64(V[k - 1].data_ptr(), w.data_ptr(), n,
                                          bc.data_ptr() + 16 * (k - 1), -1.0, None, 1.0, sp),
                       "zaxpby")
        for cc in (c1, c2):
            _lib.check(lib.tnk_zmultidot_f64(V.data_ptr(), n, k + 1, w.data_ptr(), n,
                                             cc.data_ptr(), red.data_ptr(), sp), "zmultidot")
            _lib.check(lib.tnk_zgemv_sub_f64(V.data_ptr(), n, k + 1, cc.data_ptr(),
                                             w.data_ptr(), n, sp), "zgemv_sub")
            if cc is c1:
                alph[k:k + 1].copy_(c1[2 * k:2 * k + 1])   # Re <V_k, w>: the Lanczos alpha
        if k < m - 1:
            _lib.check(lib.tnk_nrm2_f64(_real(w).data_ptr(), 2 * n, bc.data_ptr() + 16 * k,
                                        red.data_ptr(), sp), "nrm2")
            bc[2 * k:2 * k + 1].clamp_(min=1e-200)
            _lib.check(lib.tnk_scale_div_f64(_real(w).data_ptr(), _real(V[k + 1]).data_ptr(),
                                             2 * n, bc.data_ptr() + 16 * k, 1.0, sp),
                       "scale_div")
    e = bc[0:2 * (m - 1):2].reshape(1, -1) if m > 1 else None
    lam, Z = tridiag_eigh_batched(alph.reshape(1, -1), e, check=False)
    lam, Z = lam[0], Z[0]
    ph = torch.exp(torch.as_tensor(complex(tau), dtype=torch.complex128, device=dev) *
                   lam.to(torch.complex128))
    Zc = Z.to(torch.complex128)
    coef = beta0.to(torch.complex128) * (Zc @ (ph * Zc[0, :]))
    cneg = torch.view_as_real(-coef).reshape(-1).contiguous()
    out = torch.zeros(n, dtype=torch.complex128, device=dev)
    _lib.check(lib.tnk_zgemv_sub_f64(V.data_ptr(), n, m, cneg.data_ptr(), out.data_ptr(), n,
                                     sp), "zgemv_sub")
    if info is not None:
        info.update(krylov_dim=m, err_est=float("nan"), beta1=float("nan"),
                    est_ref=float("nan"), est_ref_j=0, capped=False)
    return out