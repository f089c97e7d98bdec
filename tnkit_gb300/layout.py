"""Block layouts of abelian (U(1), U(1)^n) block-sparse tensors: host metadata only.

A `Layout` is the reference's canonical `Struct` (tnkit/blocks.py:243-252): every allowed block
-- one sector per leg whose signed charges add up to the total charge -- in lexicographic sector
order, each packed row-major, one after the other in a flat buffer. Keeping this layout exactly
is what makes the GB300 kernels a drop-in: they read and write the reference's flat buffers in
place, with the block offsets and shapes computed here.

Charges are integers (U(1)) or tuples of integers (products of U(1)s, sorted lexicographically,
as tnkit/symmetry.py:169-240 orders them). The allowed blocks are found with one broadcast sum of
charges over all sector tuples, whose C-order nonzeros are already lexicographic.
"""
from __future__ import annotations

from dataclasses import dataclass
from functools import lru_cache
from typing import Dict, Sequence, Tuple

import numpy as np


def _label_array(charges) -> np.ndarray:
    """Charges as an int64 array (n_sectors, n_factors)."""
    a = np.asarray(charges, dtype=np.int64)
    return a.reshape(len(charges), -1) if a.size else np.zeros((0, 1), np.int64)


@dataclass(frozen=True)
class Leg:
    """The sectors of one leg: sorted distinct charges, their dims, and the sign (+1/-1) with
    which the leg enters charge conservation (reference `Leg`, tnkit/blocks.py:79-99)."""
    charges: Tuple
    dims: Tuple[int, ...]
    sign: int = 1

    def __post_init__(self):
        if len(self.charges) != len(self.dims) or any(int(d) < 1 for d in self.dims):
            raise ValueError(f"invalid leg {self}")
        if self.sign not in (1, -1):
            raise ValueError(f"leg sign must be +1 or -1, got {self.sign}")

    @staticmethod
    def of(x) -> "Leg":
        """A Leg from any object with charges/dims/sign (e.g. a reference `tnkit.blocks.Leg`)."""
        if isinstance(x, Leg):
            return x
        ch = tuple(tuple(int(v) for v in c) if isinstance(c, (tuple, list)) else int(c)
                   for c in x.charges)
        return Leg(ch, tuple(int(d) for d in x.dims), int(x.sign))

    @property
    def size(self) -> int:
        return int(sum(self.dims))

    def flip(self) -> "Leg":
        return Leg(self.charges, self.dims, -self.sign)

    @property
    def q(self) -> np.ndarray:
        return _label_array(self.charges)

    def starts(self) -> np.ndarray:
        d = np.asarray(self.dims, np.int64)
        return np.cumsum(d) - d

    def index_of(self, charge) -> int:
        return self.charges.index(charge)


class Layout:
    """Canonical block layout of legs `legs` and total charge `charge`.

    blocks  : (nb, nlegs) int64 sector indices, lexicographic
    shapes  : (nb, nlegs) int64 block shapes
    offsets : (nb,) int64 element offsets in the flat buffer
    size    : total elements
    """

    def __init__(self, legs: Sequence[Leg], charge):
        self.legs = tuple(Leg.of(l) for l in legs)
        self.charge = charge
        nl = len(self.legs)
        qs = [l.q * l.sign for l in self.legs]
        nf = max(q.shape[1] for q in qs) if qs else 1
        target = np.asarray(charge, np.int64).reshape(-1)
        if target.size == 1 and nf > 1:
            target = np.repeat(target, nf)
        ok = None
        for f in range(nf):
            tot = np.zeros((), np.int64)
            for i, q in enumerate(qs):
                shp = [1] * nl
                shp[i] = q.shape[0]
                tot = tot + q[:, f].reshape(shp)
            eq = tot == target[f]
            ok = eq if ok is None else (ok & eq)
        if nl == 0:
            self.blocks = np.zeros((1 if (target == 0).all() else 0, 0), np.int64)
        else:
            self.blocks = np.stack(np.nonzero(ok), axis=1).astype(np.int64)
        self.shapes = np.zeros_like(self.blocks)
        for i, l in enumerate(self.legs):
            self.shapes[:, i] = np.asarray(l.dims, np.int64)[self.blocks[:, i]]
        sizes = self.shapes.prod(1) if nl else np.ones(len(self.blocks), np.int64)
        self.sizes = sizes
        self.offsets = np.cumsum(sizes) - sizes
        self.size = int(sizes.sum())
        self._index = None
        # plain-Python views for the planners' inner loops
        self.keys = [tuple(b) for b in self.blocks.tolist()]
        self.shapes_t = [tuple(b) for b in self.shapes.tolist()]
        self.offsets_l = self.offsets.tolist()

    @property
    def nblocks(self) -> int:
        return int(self.blocks.shape[0])

    @property
    def index(self) -> Dict[Tuple[int, ...], int]:
        if self._index is None:
            self._index = {b: k for k, b in enumerate(self.keys)}
        return self._index

    def key(self, k: int) -> Tuple[int, ...]:
        return self.keys[k]

    def shape(self, k: int) -> Tuple[int, ...]:
        return self.shapes_t[k]

    def __repr__(self):
        return (f"Layout(dims={[l.size for l in self.legs]}, charge={self.charge}, "
                f"blocks={self.nblocks}, size={self.size})")


@lru_cache(maxsize=4096)
def canonical(legs: Tuple[Leg, ...], charge) -> Layout:
    """The interned canonical layout of `legs` and `charge` (one object per content)."""
    return Layout(legs, charge)


def layout_of(legs, charge) -> Layout:
    return canonical(tuple(Leg.of(l) for l in legs), charge)


def to_dense_np(layout: Layout, data: np.ndarray) -> np.ndarray:
    """Dense array (legs in sector order) of a flat host buffer: for tests and the MPO."""
    out = np.zeros(tuple(l.size for l in layout.legs), dtype=data.dtype)
    starts = [l.starts() for l in layout.legs]
    for k in range(layout.nblocks):
        b, shp, o = layout.blocks[k], layout.shape(k), int(layout.offsets[k])
        sl = tuple(slice(int(starts[i][s]), int(starts[i][s]) + shp[i]) for i, s in enumerate(b))
        out[sl] = data[o:o + int(np.prod(shp))].reshape(shp)
    return out


def from_dense_np(layout: Layout, x: np.ndarray) -> np.ndarray:
    """Flat buffer of the allowed blocks of a dense host array (legs in sector order)."""
    out = np.empty(layout.size, dtype=x.dtype)
    starts = [l.starts() for l in layout.legs]
    for k in range(layout.nblocks):
        b, shp, o = layout.blocks[k], layout.shape(k), int(layout.offsets[k])
        sl = tuple(slice(int(starts[i][s]), int(starts[i][s]) + shp[i]) for i, s in enumerate(b))
        out[o:o + int(np.prod(shp))] = x[sl].reshape(-1)
    return out
