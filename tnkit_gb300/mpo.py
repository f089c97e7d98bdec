"""Block MPOs and random block MPSs, with the reference's conventions.

  mpo_charges       tnkit/block_backend.py:162-208  (channel charges along the chain)
  to_block_mpo      tnkit/block_backend.py:211-256  (legs (wl, wr, s, s'), signs (+1,-1,+1,-1))
  random_block_mps  tnkit/block_backend.py:259-311  (bond sectors, numpy RNG, canonical order)

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


def _u1_leg(q, sign=1):
    q = np.asarray(q, dtype=np.int64)
    c, n = np.unique(q, return_counts=True)
    return (Leg(tuple(int(x) for x in c), tuple(int(x) for x in n), sign),
            np.argsort(q, kind="stable"))


def mpo_charges(mpo: Sequence[np.ndarray], site_charges, tol: float = 0.0):
    """U(1) charge of every MPO channel, one int array per MPO bond (left boundary trivial).
    Channels no nonzero path connects to both ends get charge 0 (they carry nothing)."""
    nz = [(np.abs(np.asarray(W)) > tol).any(axis=(2, 3)) for W in mpo]
    fwd = [np.ones(nz[0].shape[0], bool)]
    for m in nz:
        fwd.append(m[fwd[-1]].any(0))
    bwd = [np.ones(nz[-1].shape[1], bool)]
    for m in reversed(nz):
        bwd.append(m[:, bwd[-1]].any(1))
    live = [f & b for f, b in zip(fwd, reversed(bwd))]
    out = [np.zeros(np.shape(mpo[0])[0], np.int64)]
    for n, (W, q) in enumerate(zip(mpo, site_charges)):
        W = np.asarray(W)
        a, b, s, t = np.nonzero(np.abs(W) > tol)
        keep = live[n][a] & live[n + 1][b]
        vals = out[-1][a[keep]] + np.asarray(q)[s[keep]] - np.asarray(q)[t[keep]]
        qr = np.zeros(W.shape[1], np.int64)
        for j in np.flatnonzero(live[n + 1]):
            v = np.unique(vals[b[keep] == j])
            if len(v) != 1:
                raise ValueError(f"MPO site {n}, right channel {j}: charges {v.tolist()} "
                                 "(write the terms with charged operators such as S+ S-)")
            qr[j] = v[0]
        out.append(qr)
    return out


def to_block_mpo(mpo: Sequence[np.ndarray], site_charges, device="cuda", tol: float = 0.0):
    """A dense MPO as block tensors (U(1)); returns (tensors, orders) like the reference."""
    chans = mpo_charges(mpo, site_charges, tol)
    out, orders = [], []
    for n, W in enumerate(mpo):
        W = np.asarray(W)
        if np.iscomplexobj(W):
            if np.abs(W.imag).max() > 1e-12 * max(1.0, np.abs(W.real).max()):
                raise TypeError("complex MPO entries need a complex backend")
            W = W.real
        (cl, ol), (cr, orr) = _u1_leg(chans[n]), _u1_leg(chans[n + 1])
        p, op = _u1_leg(site_charges[n])
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


def random_block_mps(mpo: Sequence[BlockTensor], chi: int, charge: int, rng,
                     device="cuda") -> List[BlockTensor]:
    """Random block MPS of total charge `charge`, bonds of at most `chi` states, drawn from `rng`
    in the reference's order (one standard_normal(size) per site, canonical layout)."""
    phys = [W.legs[2] for W in mpo]

    def grow(counts, leg, sign):
        out = {}
        for c, n in counts.items():
            for a, d in zip(leg.charges, leg.dims):
                c2 = c + (a if sign > 0 else -a)
                out[c2] = out.get(c2, 0) + n * d
        return out

    left, right = [{0: 1}], [{charge: 1}]
    for p in phys:
        left.append(grow(left[-1], p, 1))
    for p in reversed(phys):
        right.append(grow(right[-1], p, -1))
    right.reverse()
    if charge not in left[-1]:
        raise ValueError(f"no state of these sites has total charge {charge!r}")
    bonds, cand = [], {0}
    for n, (lc, rc) in enumerate(zip(left, right)):
        w = {c: min(lc[c], rc[c]) for c in cand if c in rc}
        keep = sorted(w, key=lambda c: (-w[c], c))[:chi]
        tot = sum(w[c] for c in keep)
        dims = {c: min(w[c], max(1, int(chi * w[c] / tot))) for c in keep}
        while sum(dims.values()) > chi:
            dims[max(dims, key=dims.get)] -= 1
        bonds.append(dims)
        if n < len(phys):
            cand = {c + a for c in keep for a in phys[n].charges}
    for n in range(len(phys) - 1, -1, -1):
        prv = {c - a for c in bonds[n + 1] for a in phys[n].charges}
        bonds[n] = {c: d for c, d in bonds[n].items() if c in prv}
    legs = [Leg(tuple(sorted(b)), tuple(b[c] for c in sorted(b)), 1) for b in bonds]
    out = []
    for n, p in enumerate(phys):
        lay = layout_of((legs[n], p, legs[n + 1].flip()), 0)
        host = rng.standard_normal((lay.size,))
        out.append(BlockTensor(lay, torch.as_tensor(host, device=device)))
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
