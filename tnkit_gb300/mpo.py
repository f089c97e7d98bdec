"""Block MPOs and random block MPSs, with the reference's conventions.

  mpo_charges       tnkit/block_backend.py:162-208  (channel charges along the chain)
  to_block_mpo      tnkit/block_backend.py:211-256  (legs (wl, wr, s, s'), signs (+1,-1,+1,-1))
  random_block_mps  tnkit/block_backend.py:259-311  (bond sectors, numpy RNG, canonical order)

Charges are U(1) ints or, for a product of U(1)s (the (N_up, N_down) labels of the Hubbard
chain), tuples sorted lexicographically with the first factor most significant, as the
reference's ProductSymmetry orders them (tnkit/symmetry.py:169-240).

These run on the host once per problem; the results are uploaded to the GPU. The random MPS
draws the same numbers from the same generator as the reference, so a seeded run starts from
the reference's own initial state.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np
import torch

from .layout import Leg, layout_of, from_dense_np
from .tensor import BlockTensor


def _label_rows(q):
    """Charges as an int array (n, factors) and whether they are tuples (a product of U(1)s)."""
    a = np.asarray(q, dtype=np.int64)
    if a.ndim == 1:
        return a.reshape(-1, 1), False
    return a.reshape(len(a), -1), True


def _as_label(row, product: bool):
    return tuple(int(v) for v in row) if product else int(row[0])


def _leg_from_charges(q, sign=1):
    """The leg whose dense index i has charge q[i], and the dense indices in sector order (stable
    within a sector); sectors sorted lexicographically, the first factor most significant
    (tnkit/blocks.py:104-118, tnkit/symmetry.py:169-240)."""
    a, product = _label_rows(q)
    uniq, inv, counts = np.unique(a, axis=0, return_inverse=True, return_counts=True)
    return (Leg(tuple(_as_label(r, product) for r in uniq), tuple(int(n) for n in counts), sign),
            np.argsort(np.ravel(inv), kind="stable"))


def mpo_charges(mpo: Sequence[np.ndarray], site_charges, tol: float = 0.0):
    """The charge of every MPO channel, one array per MPO bond (left boundary trivial): int
    arrays for U(1) site charges, (channels, factors) arrays for tuple charges (U(1) x U(1) ...).
    Channels no nonzero path connects to both ends get the trivial charge (they carry nothing)."""
    nz = [(np.abs(np.asarray(W)) > tol).any(axis=(2, 3)) for W in mpo]
    fwd = [np.ones(nz[0].shape[0], bool)]
    for m in nz:
        fwd.append(m[fwd[-1]].any(0))
    bwd = [np.ones(nz[-1].shape[1], bool)]
    for m in reversed(nz):
        bwd.append(m[:, bwd[-1]].any(1))
    live = [f & b for f, b in zip(fwd, reversed(bwd))]
    q0, product = _label_rows(site_charges[0])
    nf = q0.shape[1]
    out = [np.zeros((np.shape(mpo[0])[0], nf), np.int64)]
    for n, (W, q) in enumerate(zip(mpo, site_charges)):
        W = np.asarray(W)
        qa, _ = _label_rows(q)
        a, b, s, t = np.nonzero(np.abs(W) > tol)
        keep = live[n][a] & live[n + 1][b]
        vals = out[-1][a[keep]] + qa[s[keep]] - qa[t[keep]]
        bk = b[keep]
        qr = np.zeros((W.shape[1], nf), np.int64)
        for j in np.flatnonzero(live[n + 1]):
            v = np.unique(vals[bk == j], axis=0)
            if len(v) != 1:
                raise ValueError(f"MPO site {n}, right channel {j}: charges {v.tolist()} "
                                 "(write the terms with charged operators such as S+ S-)")
            qr[j] = v[0]
        out.append(qr)
    return out if product else [c[:, 0].copy() for c in out]


def to_block_mpo(mpo: Sequence[np.ndarray], site_charges, device="cuda", tol: float = 0.0):
    """A dense MPO as block tensors under U(1) (int site charges) or a product of U(1)s (tuple
    site charges, e.g. (N_up, N_down)); returns (tensors, orders) like the reference
    (tnkit/block_backend.py:211-256)."""
    chans = mpo_charges(mpo, site_charges, tol)
    out, orders = [], []
    for n, W in enumerate(mpo):
        W = np.asarray(W)
        if np.iscomplexobj(W):
            if np.abs(W.imag).max() > 1e-12 * max(1.0, np.abs(W.real).max()):
                raise TypeError("complex MPO entries need a complex backend")
            W = W.real
        (cl, ol), (cr, orr) = _leg_from_charges(chans[n]), _leg_from_charges(chans[n + 1])
        p, op = _leg_from_charges(site_charges[n])
        x = W.astype(np.float64)
        for i, o in enumerate((ol, orr, op, op)):
            x = np.take(x, o, axis=i)
        lay = layout_of((cl, cr.flip(), p, p.flip()), 0)
        host = from_dense_np(lay, x)
        out.append(BlockTensor(lay, torch.as_tensor(host, device=device), host))
        orders.append((ol, orr, op, op))
    return out, orders


def dense_mpo(mpo: Sequence[np.ndarray], device="cuda"):
    """A dense MPO as one-block tensors (trivial charges), for the dense path."""
    out = []
    for W in mpo:
        W = np.ascontiguousarray(np.real_if_close(np.asarray(W)), dtype=np.float64)
        wl, wr, d, _ = W.shape
        lay = layout_of((Leg((0,), (wl,), 1), Leg((0,), (wr,), -1), Leg((0,), (d,), 1),
                         Leg((0,), (d,), -1)), 0)
        host = W.reshape(-1).copy()
        out.append(BlockTensor(lay, torch.as_tensor(host, device=device), host))
    return out


def _fuse(a, b, sign=1):
    if isinstance(a, tuple):
        return tuple(x + sign * y for x, y in zip(a, b))
    return a + sign * b


def random_block_mps(mpo: Sequence[BlockTensor], chi: int, charge, rng,
                     device="cuda") -> List[BlockTensor]:
    """Random block MPS of total charge `charge` (an int, or a tuple for a product of U(1)s),
    bonds of at most `chi` states, drawn from `rng` in the reference's order (one
    standard_normal(size) per site, canonical layout; tnkit/block_backend.py:259-311)."""
    phys = [W.legs[2] for W in mpo]
    product = isinstance(phys[0].charges[0], tuple)
    if product:
        charge = tuple(int(c) for c in charge)
        unit = tuple(0 for _ in phys[0].charges[0])
    else:
        unit = 0

    def grow(counts, leg, sign):
        out = {}
        for c, n in counts.items():
            for a, d in zip(leg.charges, leg.dims):
                c2 = _fuse(c, a, 1 if sign > 0 else -1)
                out[c2] = out.get(c2, 0) + n * d
        return out

    left, right = [{unit: 1}], [{charge: 1}]
    for p in phys:
        left.append(grow(left[-1], p, 1))
    for p in reversed(phys):
        right.append(grow(right[-1], p, -1))
    right.reverse()
    if charge not in left[-1]:
        raise ValueError(f"no state of these sites has total charge {charge!r}")
    bonds, cand = [], {unit}
    for n, (lc, rc) in enumerate(zip(left, right)):
        w = {c: min(lc[c], rc[c]) for c in cand if c in rc}
        keep = sorted(w, key=lambda c: (-w[c], c))[:chi]
        tot = sum(w[c] for c in keep)
        dims = {c: min(w[c], max(1, int(chi * w[c] / tot))) for c in keep}
        while sum(dims.values()) > chi:
            dims[max(dims, key=dims.get)] -= 1
        bonds.append(dims)
        if n < len(phys):
            cand = {_fuse(c, a) for c in keep for a in phys[n].charges}
    for n in range(len(phys) - 1, -1, -1):
        prv = {_fuse(c, a, -1) for c in bonds[n + 1] for a in phys[n].charges}
        bonds[n] = {c: d for c, d in bonds[n].items() if c in prv}
    legs = [Leg(tuple(sorted(b)), tuple(b[c] for c in sorted(b)), 1) for b in bonds]
    out = []
    for n, p in enumerate(phys):
        lay = layout_of((legs[n], p, legs[n + 1].flip()), unit)
        host = rng.standard_normal((lay.size,))
        out.append(BlockTensor(lay, torch.as_tensor(host, device=device)))
    return out


def product_block_mps(mpo: Sequence[BlockTensor], states: Sequence[int],
                      device="cuda") -> List[BlockTensor]:
    """The product state with site n in the physical sector of charge `states[n]` (e.g. the Neel
    state of a spin-1/2 S^z chain, charges +1 -1 +1 ...): bonds of one state each, the left
    bond of site n carrying the charge of sites 0 .. n-1, every site one block holding 1. The
    physical sectors must be one-dimensional."""
    out = []
    q = 0
    for W, s in zip(mpo, states):
        p = W.legs[2]
        if s not in p.charges or p.dims[p.charges.index(s)] != 1:
            raise ValueError(f"charge {s!r} is not a one-dimensional physical sector")
        lay = layout_of((Leg((q,), (1,), 1), p, Leg((q + s,), (1,), -1)), 0)
        out.append(BlockTensor(lay, torch.ones(lay.size, dtype=torch.float64, device=device)))
        q += s
    return out


def random_dense_mps(N: int, chi: int, d: int, rng, device="cuda") -> List[BlockTensor]:
    """Dense random MPS drawn as the reference's `random_mps` (tnkit/_dmrg.py:253-261)."""
    dims = [1] + [min(chi, d ** min(i, N - i)) for i in range(1, N)] + [1]
    out = []
    for i in range(N):
        x = rng.standard_normal((dims[i], d, dims[i + 1]))
        lay = layout_of((Leg((0,), (dims[i],), 1), Leg((0,), (d,), 1),
                         Leg((0,), (dims[i + 1],), -1)), 0)
        out.append(BlockTensor(lay, torch.as_tensor(x.reshape(-1), device=device)))
    return out
