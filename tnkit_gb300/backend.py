"""The `backend="b200"` adaptor: the reference's backend interface (tnkit/backend.py:491-816) on
the GPU, with the hot path routed to the tnk_* kernels.

`get_backend("b200")` returns a complex128 `B200Backend` and `get_backend("b200-real")` a float64
one, as the reference's 'torch-cuda' / 'torch-cuda-real' pair; 'b200-ff', 'b200-mixed' and
'b200-mixed-ff' are float64 backends whose DMRG runs the float-float or tensor-core Lanczos.
The dense methods keep the reference's names, arguments and return types on CUDA torch tensors;
they are the small glue of the reference's solvers (Krylov projected problems, norms, casts),
not the hot path. The hot path -- two-site and one-site H_eff, left and right environment
updates, block tensordot, the DMRG / TDVP sweeps -- takes this package's block tensors and runs in
the library, and so does the Krylov-exponential step of the dense interface
(`expm_sym_tridiag_eigh`, whose tridiagonal eigenproblem is a hand-written kernel). In a process
that imports the reference package, `tnkit_gb300.frontdoor.install()` makes the reference's own
`dmrg` / `tdvp2_evolve` / `get_backend` accept these backends.

There is no fallback: on a host without CUDA the hot methods raise.
"""
from __future__ import annotations

import os
from typing import Any, Optional

import numpy as np

_SPECS = {"b200": ("complex", "f64"), "b200-real": ("real", "f64"), "b200-ff": ("real", "ff"),
          "b200-mixed": ("real", "mixed"), "b200-mixed-ff": ("real", "mixed-ff")}


class B200Backend:
    is_torch = True

    def __init__(self, device: Optional[str] = None, precision: str = "f64",
                 complex: bool = False):
        import torch
        self.torch = torch
        self._device = device
        if precision not in ("f64", "ff", "mixed", "mixed-ff"):
            raise ValueError("precision must be 'f64', 'ff', 'mixed' or 'mixed-ff'")
        if complex and precision != "f64":
            raise ValueError("the complex backend computes in complex128 (precision 'f64')")
        self.precision = precision
        self.is_complex = bool(complex)
        self.dtype = torch.complex128 if complex else torch.float64
        self.rdtype = torch.float64
        self.name = "b200" if complex else ("b200-real" if precision == "f64"
                                            else f"b200-{precision}")

    @classmethod
    def from_spec(cls, spec: str, device: Optional[str] = None) -> "B200Backend":
        if spec not in _SPECS:
            raise ValueError(f"unknown backend {spec!r}; this package provides "
                             f"{', '.join(repr(s) for s in _SPECS)}")
        kind, prec = _SPECS[spec]
        return cls(device=device, precision=prec, complex=kind == "complex")

    @property
    def device(self):
        t = self.torch
        if self._device is not None:
            return t.device(self._device)
        if not t.cuda.is_available():
            raise RuntimeError("backend 'b200' needs a CUDA device (GB300)")
        return t.device("cuda", t.cuda.current_device())

    # --- array creation / movement (tnkit/backend.py:510-579) ---
    def _check_real(self, im, re):
        m = float(abs(im).max()) if im.numel() else 0.0
        r = float(abs(re).max()) if re.numel() else 1.0
        if m > 1e-12 * max(1.0, r):
            raise TypeError(f"backend {self.name!r} is real: the array has an imaginary part "
                            f"(max|imag| = {m:.3e})")

    def array(self, x):
        t = self.torch
        if not isinstance(x, t.Tensor):
            a = np.asarray(x)
            x = t.as_tensor(a)
        if not self.is_complex and t.is_complex(x):
            self._check_real(x.imag, x.real)
            x = x.real
        return x.to(self.device, self.dtype)

    def to_numpy(self, x):
        x = x.detach()
        if x.is_conj():
            x = x.resolve_conj()
        if x.is_neg():
            x = x.resolve_neg()
        return x.cpu().numpy()

    def randn(self, rng, shape):
        r = rng.standard_normal(shape)
        if self.is_complex:
            r = r + 1j * rng.standard_normal(shape)
        return self.array(r)

    def zeros(self, shape):
        return self.torch.zeros(shape, dtype=self.dtype, device=self.device)

    def ones(self, shape):
        return self.torch.ones(shape, dtype=self.dtype, device=self.device)

    def zeros_like(self, a):
        return self.torch.zeros_like(a)

    def conj(self, a):
        return self.torch.conj(a) if self.torch.is_complex(a) else a

    def transpose(self, x, perm):
        return x.permute(*perm)

    def diag(self, v):
        return self.torch.diag(v.to(self.dtype) if v.dtype != self.dtype else v)

    def astype(self, x, which):
        """'low' / 'high': the reference casts to complex64 / complex128 (tnkit/backend.py:554);
        a real backend keeps real data real (float32 / float64)."""
        t = self.torch
        cplx = self.is_complex or t.is_complex(x)
        if which == "low":
            return x.to(t.complex64 if cplx else t.float32)
        return x.to(t.complex128 if cplx else t.float64)

    # --- reductions / scalars ---
    def vdot(self, a, b):
        return self.torch.vdot(a.reshape(-1), b.reshape(-1))

    def norm(self, a):
        return self.torch.linalg.vector_norm(a.reshape(-1))

    def to_scalar(self, x):
        return complex(x.item()) if hasattr(x, "item") else complex(x)

    def sync(self):
        self.torch.cuda.synchronize(self.device)

    def einsum(self, sub, *ops):
        return self.torch.einsum(sub, *ops)

    # --- small dense helpers of the Krylov solvers (tnkit/backend.py:599-753) ---
    def stack(self, xs):
        t = self.torch
        return t.stack([x if isinstance(x, t.Tensor) else t.as_tensor(x, device=self.device)
                        for x in xs])

    def tridiag(self, d, e):
        t = self.torch
        T = t.diag(d.to(self.dtype))
        if e is not None and int(e.shape[0]) > 0:
            e = e.to(self.dtype)
            T = T + t.diag(e, 1) + t.diag(e, -1)
        return T

    def expm(self, A):
        return self.torch.matrix_exp(A)

    def expm_host(self, A):
        from scipy.linalg import expm as _e
        return _e(self.to_numpy(A))

    def expm_sym_tridiag_eigh(self, d, e, tau):
        """exp(tau T) of the real symmetric tridiagonal T = tridiag(e, d, e) on the device, by
        T's eigendecomposition computed by the library's tridiagonal eigensolver kernel
        (tnk_tridiag_eig_f64, one launch) rather than a dense eigensolver: the reference's
        eigh route (tnkit/backend.py:643-661)."""
        out = self.expm_sym_tridiag_eigh_batched(d.reshape(1, -1),
                                                 None if e is None else e.reshape(1, -1), tau)
        return out[0]

    def expm_sym_tridiag_eigh_batched(self, d, e, tau):
        from .tridiag import tridiag_eigh_batched
        t = self.torch
        dd = (d.real if t.is_complex(d) else d).to(t.float64)
        ee = None if e is None else (e.real if t.is_complex(e) else e).to(t.float64)
        lam, V = tridiag_eigh_batched(dd, ee)
        cd = t.complex128 if (self.is_complex or isinstance(tau, complex)) else t.float64
        ph = t.exp(t.as_tensor(tau, dtype=cd, device=dd.device) * lam.to(cd))
        Vc = V.to(cd)
        return (Vc * ph.unsqueeze(-2)) @ Vc.transpose(-1, -2)

    def expm_taylor(self, A, squarings, order=18):
        t = self.torch
        As = A / (2.0 ** int(squarings))
        E = t.eye(A.shape[-1], dtype=A.dtype, device=A.device)
        term = E
        for k in range(1, int(order) + 1):
            term = (term @ As) / k
            E = E + term
        for _ in range(int(squarings)):
            E = E @ E
        return E

    def mv(self, A, x):
        return A @ x

    def vm(self, c, A):
        return c @ A

    def guard_denom(self, x, tiny=1e-200):
        return self.torch.clamp(x, min=tiny)

    def norm_axis(self, x, axis=-1):
        return self.torch.linalg.vector_norm(x, dim=axis)

    def stack_axis(self, xs, axis=-1):
        return self.torch.stack(list(xs), dim=axis)

    # --- dense linear algebra (cuSOLVER's gesvd, as the reference selects on CUDA) ---
    def svd(self, A):
        drv = os.environ.get("TNKIT_CUDA_SVD_DRIVER", "gesvd")
        return self.torch.linalg.svd(A, full_matrices=False,
                                     driver=None if drv == "default" else drv)

    def svd_batched(self, A):
        drv = os.environ.get("TNKIT_CUDA_SVD_DRIVER_BATCHED", "gesvd")
        return self.torch.linalg.svd(A, full_matrices=False,
                                     driver=None if drv == "default" else drv)

    def qr(self, A):
        return self.torch.linalg.qr(A, mode="reduced")

    def eigh(self, A):
        return self.torch.linalg.eigh(A)

    # --- the hot path on block tensors (tnkit/_dmrg.py:162-231, blocks.py:1156-1192) ---
    def apply_two_site(self, theta, L, W1, W2, R):
        from . import ops
        return ops.apply_two_site(theta, L, W1, W2, R)

    def apply_one_site(self, M, L, W, R):
        from . import ops
        return ops.apply_one_site(M, L, W, R)

    def update_left_env(self, L, A, W):
        from . import ops
        return ops.update_left_env(L, A, W)

    def update_right_env(self, R, B, W):
        from . import ops
        return ops.update_right_env(R, B, W)

    def tensordot(self, a, b, nc: int = 1):
        from . import ops
        return ops.tensordot(a, b, nc)

    def truncated_svd(self, m, chi, **kw):
        from . import linalg
        return linalg.truncated_svd(m, chi, **kw)

    def dmrg(self, mpo, chi, options=None, **kw):
        from .dmrg import dmrg
        kw.setdefault("precision", self.precision)
        return dmrg(mpo, chi, options, **kw)

    def tdvp2_evolve(self, mps, mpo, chi, dt, n_steps, **kw):
        from .tdvp import tdvp2_evolve
        return tdvp2_evolve(mps, mpo, chi, dt, n_steps, **kw)

    def __repr__(self):
        return f"B200Backend(name={self.name!r})"


def get_backend(spec: Any = "b200", **kw):
    """A `B200Backend` from its name ('b200', 'b200-real', 'b200-ff', 'b200-mixed',
    'b200-mixed-ff'); a backend object is returned unchanged (tnkit/backend.py:192-240)."""
    if not isinstance(spec, str):
        return spec
    return B200Backend.from_spec(spec, **kw)
