"""The `backend="b200"` adaptor: the reference's backend interface (tnkit/backend.py:491-816) on
the GPU, with the hot-path contractions routed to the tnk_* kernels.

`get_backend("b200")` returns a `B200Backend`. Its dense methods (array, randn, zeros, einsum,
vdot, norm, svd, qr, eigh, astype, ...) keep the reference's names and meanings on CUDA float64
torch tensors. The DMRG inner loop -- two-site and one-site H_eff, left and right environment
updates, the two-site block -- takes block tensors (`tnkit_gb300.BlockTensor`, the reference's
canonical layout) and runs in the library: `apply_two_site`, `apply_one_site`,
`update_left_env`, `update_right_env`, `tensordot`. `B200Backend.dmrg` is the sweep driver
(tnkit_gb300.dmrg.dmrg) bound to this backend.

There is no fallback: on a host without CUDA the hot methods raise.
"""
from __future__ import annotations

from typing import Any, Optional

import numpy as np


class B200Backend:
    name = "b200"
    is_torch = True
    is_complex = False

    def __init__(self, device: Optional[str] = None, precision: str = "f64"):
        import torch
        self.torch = torch
        self._device = device
        self.dtype = torch.float64
        self.rdtype = torch.float64
        if precision not in ("f64", "mixed"):
            raise ValueError("precision must be 'f64' or 'mixed'")
        self.precision = precision

    @property
    def device(self):
        t = self.torch
        if self._device is not None:
            return t.device(self._device)
        if not t.cuda.is_available():
            raise RuntimeError("backend 'b200' needs a CUDA device (GB300)")
        return t.device("cuda", t.cuda.current_device())

    # --- array creation / movement (tnkit/backend.py:524-552) ---
    def array(self, x):
        t = self.torch
        if isinstance(x, t.Tensor):
            if t.is_complex(x):
                if float(x.imag.abs().max()) > 1e-12 * max(1.0, float(x.real.abs().max())):
                    raise TypeError("backend 'b200' is real: the array has an imaginary part")
                x = x.real
            return x.to(self.device, self.dtype)
        a = np.asarray(x)
        if np.iscomplexobj(a):
            if np.abs(a.imag).max(initial=0.0) > 1e-12 * max(1.0, np.abs(a.real).max(initial=0)):
                raise TypeError("backend 'b200' is real: the array has an imaginary part")
            a = a.real
        return t.as_tensor(a, dtype=self.dtype, device=self.device)

    def to_numpy(self, x):
        return x.detach().cpu().numpy()

    def randn(self, rng, shape):
        return self.array(rng.standard_normal(shape))

    def zeros(self, shape):
        return self.torch.zeros(shape, dtype=self.dtype, device=self.device)

    def ones(self, shape):
        return self.torch.ones(shape, dtype=self.dtype, device=self.device)

    def zeros_like(self, a):
        return self.torch.zeros_like(a)

    def conj(self, a):
        return a

    def transpose(self, x, perm):
        return x.permute(*perm)

    def diag(self, v):
        return self.torch.diag(v)

    def astype(self, x, which):
        return x.to(self.torch.float32 if which == "low" else self.torch.float64)

    # --- reductions / scalars ---
    def vdot(self, a, b):
        return self.torch.dot(a.reshape(-1), b.reshape(-1))

    def norm(self, a):
        return self.torch.linalg.vector_norm(a.reshape(-1))

    def to_scalar(self, x):
        return complex(x.item()) if hasattr(x, "item") else complex(x)

    def sync(self):
        self.torch.cuda.synchronize()

    # --- dense linear algebra ---
    def einsum(self, sub, *ops):
        return self.torch.einsum(sub, *ops)

    def svd(self, a):
        return self.torch.linalg.svd(a, full_matrices=False, driver="gesvd")

    def qr(self, a):
        return self.torch.linalg.qr(a)

    def eigh(self, a):
        return self.torch.linalg.eigh(a)

    # --- the hot path on block tensors (tnkit/_dmrg.py:162-231) ---
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

    def dmrg(self, mpo, chi, options=None, **kw):
        from .dmrg import dmrg
        kw.setdefault("precision", self.precision)
        return dmrg(mpo, chi, options, **kw)

    def __repr__(self):
        return f"B200Backend(precision={self.precision!r})"


def get_backend(spec: Any = "b200", **kw):
    """`get_backend("b200")` (also "b200-mixed") -> B200Backend; a backend object is returned
    unchanged (tnkit/backend.py:192-240)."""
    if not isinstance(spec, str):
        return spec
    if spec in ("b200", "b200-real"):
        return B200Backend(**kw)
    if spec == "b200-mixed":
        return B200Backend(precision="mixed", **kw)
    raise ValueError(f"unknown backend {spec!r}; this package provides 'b200' and 'b200-mixed'")
