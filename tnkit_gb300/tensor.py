"""The product's block tensor: a canonical `Layout` and one flat buffer.

Same contract as the reference's `BlockTensor(struct, data)` (tnkit/blocks.py:697-760): `data` is
a 1-D contiguous buffer of length `layout.size` holding every allowed block in canonical order.
Device tensors (torch, CUDA, float64) are the working form; MPO tensors also keep a host copy,
because their entries become scalar coefficients of the kernel plans.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .layout import Layout, Leg, layout_of, to_dense_np


class BlockTensor:
    __slots__ = ("layout", "data", "host")
    is_block = True

    def __init__(self, layout: Layout, data, host: Optional[np.ndarray] = None):
        n = int(data.shape[0]) if hasattr(data, "shape") else len(data)
        if n != layout.size or len(getattr(data, "shape", (n,))) != 1:
            raise ValueError(f"buffer of {tuple(getattr(data, 'shape', (n,)))} for a layout of "
                             f"size {layout.size}")
        self.layout, self.data, self.host = layout, data, host

    @property
    def legs(self):
        return self.layout.legs

    @property
    def charge(self):
        return self.layout.charge

    @property
    def shape(self):
        return tuple(l.size for l in self.layout.legs)

    @property
    def ndim(self):
        return len(self.layout.legs)

    def numpy(self) -> np.ndarray:
        if self.host is not None:
            return self.host
        return self.data.detach().cpu().numpy()

    def to_dense(self) -> np.ndarray:
        """Dense host array, legs in sector order."""
        return to_dense_np(self.layout, self.numpy())

    def with_data(self, data) -> "BlockTensor":
        return BlockTensor(self.layout, data)

    def __repr__(self):
        return f"BlockTensor({self.layout})"

    @staticmethod
    def from_reference(t, device="cuda", dtype=None) -> "BlockTensor":
        """This package's tensor of a reference `tnkit.blocks.BlockTensor` (any struct; laid out
        canonically by the reference's own `.canonical()` first): the same canonical buffer,
        block for block, moved to `device`. Real data become float64 and complex data
        complex128 unless `dtype` is given; a real tensor also keeps its host copy (MPO tensors'
        entries become plan coefficients)."""
        import torch
        c = t.canonical()
        lay = layout_of([Leg.of(l) for l in c.struct.legs], c.struct.charge)
        d = c.data
        x = d.detach() if isinstance(d, torch.Tensor) else torch.as_tensor(np.asarray(d))
        if dtype is None:
            dtype = torch.complex128 if torch.is_complex(x) else torch.float64
        x = x.to(dtype=dtype).contiguous()
        host = None if torch.is_complex(x) else x.cpu().numpy()
        return BlockTensor(lay, x.to(device), host)


def dense_layout(shape: Sequence[int], signs: Sequence[int]) -> Layout:
    """The one-block layout of a dense tensor (trivial charge on every leg)."""
    return layout_of([Leg((0,), (int(n),), int(s)) for n, s in zip(shape, signs)], 0)
