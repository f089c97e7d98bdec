"""Small real symmetric tridiagonal eigenproblems on the GPU (tnk_tridiag_eig_f64): the
projected problems of the Krylov solvers, solved next to their coefficients.

  tridiag_eigh_batched(d, e)   d (k, m), e (k, m-1) float64 CUDA -> lam (k, m) ascending,
                               V (k, m, m) with eigenvectors in the columns; the decomposition
                               behind the reference's expm_sym_tridiag_eigh(_batched)
                               (tnkit/backend.py:643-661, :729-751)
"""
from __future__ import annotations

from typing import Optional

import torch

from . import _lib


def tridiag_eigh_batched(d: torch.Tensor, e: Optional[torch.Tensor], check: bool = True,
                         info: Optional[torch.Tensor] = None):
    """Eigendecomposition of each tridiag(e[b], d[b], e[b]) in one launch. With check=True the
    convergence flags are read back (one synchronisation) and a failure raises; with
    check=False they are left in `info` (an int32 CUDA tensor of k entries, allocated when not
    given) for the caller to read when it synchronises anyway."""
    if d.dim() != 2 or not d.is_cuda or d.dtype != torch.float64:
        raise TypeError("d must be a (k, m) float64 CUDA tensor")
    k, m = (int(x) for x in d.shape)
    if m < 1 or m > _lib.TNK_TRIDIAG_MAX_N:
        raise ValueError(f"order {m} outside [1, {_lib.TNK_TRIDIAG_MAX_N}]")
    d = d.contiguous()
    if m > 1:
        if e is None or tuple(e.shape) != (k, m - 1) or e.dtype != torch.float64 or not e.is_cuda:
            raise TypeError("e must be a (k, m-1) float64 CUDA tensor")
        e = e.contiguous()
    lam = torch.empty((k, m), dtype=torch.float64, device=d.device)
    V = torch.empty((k, m, m), dtype=torch.float64, device=d.device)
    if info is None:
        info = torch.empty(k, dtype=torch.int32, device=d.device)
    lib = _lib.lib()
    _lib.check(lib.tnk_tridiag_eig_f64(d.data_ptr(), e.data_ptr() if m > 1 else None, m, k, m,
                                       max(m - 1, 1), lam.data_ptr(), V.data_ptr(),
                                       info.data_ptr(), _lib.stream_ptr()), "tridiag_eig")
    if check and k:
        bad = int(info.max().item())
        if bad:
            raise RuntimeError(f"tridiagonal eigensolver: eigenvalue {bad - 1} did not converge")
    return lam, V
