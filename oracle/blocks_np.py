"""Block-sparse U(1) tensors for the oracle (numpy, CPU; test infrastructure only).

Restates the layout and algebra of the reference's `tnkit/blocks.py` in a deliberately simple
form: blocks are held in a dict keyed by sector tuples, and a contraction loops over block pairs.
The canonical flat layout -- every allowed block in lexicographic sector order, each packed
row-major (reference `tnkit/blocks.py:243-252`) -- is reproduced exactly, so flat buffers compare
one to one with the reference's and with the product's.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass
from typing import Dict, List, Sequence, Tuple

import numpy as np


@dataclass(frozen=True)
class Leg:
    """Sectors of one leg: sorted distinct integer charges, their dims, and the sign (+1/-1)
    with which the leg enters charge conservation (reference `tnkit/blocks.py:79-99`)."""
    charges: Tuple[int, ...]
    dims: Tuple[int, ...]
    sign: int = 1

    @property
    def size(self) -> int:
        return int(sum(self.dims))

    def flip(self) -> "Leg":
        return Leg(self.charges, self.dims, -self.sign)

    @staticmethod
    def from_json(d) -> "Leg":
        return Leg(tuple(int(c) for c in d["charges"]), tuple(int(x) for x in d["dims"]),
                   int(d["sign"]))


def allowed(legs: Sequence[Leg], charge: int) -> List[Tuple[int, ...]]:
    """Allowed sector tuples in lexicographic order: signed charges sum to `charge`
    (reference `tnkit/blocks.py:199-225`, `canonical` `:243-252`)."""
    out = []
    for t in itertools.product(*(range(len(l.charges)) for l in legs)):
        if sum(l.sign * l.charges[s] for l, s in zip(legs, t)) == charge:
            out.append(t)
    return out


class BT:
    """A block tensor: legs, total charge and a dict {sector tuple: dense block}. Every allowed
    block is present (zeros where nothing was written)."""

    def __init__(self, legs, charge, blocks=None, dtype=np.float64):
        self.legs = tuple(legs)
        self.charge = int(charge)
        self.keys = allowed(self.legs, self.charge)
        self.blocks: Dict[Tuple[int, ...], np.ndarray] = {}
        for k in self.keys:
            shp = self.shape_of(k)
            if blocks is not None and k in blocks:
                self.blocks[k] = np.asarray(blocks[k]).reshape(shp)
            else:
                self.blocks[k] = np.zeros(shp, dtype)

    def shape_of(self, k):
        return tuple(l.dims[s] for l, s in zip(self.legs, k))

    @property
    def size(self) -> int:
        return int(sum(int(np.prod(self.shape_of(k))) for k in self.keys))

    @property
    def dtype(self):
        for b in self.blocks.values():
            return b.dtype
        return np.float64

    # --- canonical flat buffer (reference `tnkit/blocks.py:243-252`) ---
    def flat(self) -> np.ndarray:
        if not self.keys:
            return np.zeros(0)
        return np.concatenate([self.blocks[k].reshape(-1) for k in self.keys])

    @staticmethod
    def from_flat(legs, charge, data) -> "BT":
        t = BT(legs, charge, dtype=np.asarray(data).dtype)
        data = np.asarray(data)
        o = 0
        for k in t.keys:
            shp = t.shape_of(k)
            n = int(np.prod(shp))
            t.blocks[k] = data[o:o + n].reshape(shp).copy()
            o += n
        if o != data.size:
            raise ValueError(f"buffer of {data.size} entries for a layout of {o}")
        return t

    @staticmethod
    def from_json(meta, data) -> "BT":
        return BT.from_flat([Leg.from_json(l) for l in meta["legs"]], meta["charge"], data)

    def to_dense(self) -> np.ndarray:
        """Dense array with every leg in sector order."""
        starts = [np.concatenate([[0], np.cumsum(l.dims)[:-1]]).astype(int) for l in self.legs]
        out = np.zeros(tuple(l.size for l in self.legs), self.dtype)
        for k in self.keys:
            sl = tuple(slice(starts[i][s], starts[i][s] + self.legs[i].dims[s])
                       for i, s in enumerate(k))
            out[sl] = self.blocks[k]
        return out

    # --- algebra ---
    def transpose(self, perm) -> "BT":
        perm = tuple(perm)
        return BT([self.legs[p] for p in perm], self.charge,
                  {tuple(k[p] for p in perm): np.transpose(b, perm)
                   for k, b in self.blocks.items()}, self.dtype)

    def conj(self) -> "BT":
        """The dual: signs and total charge flipped, entries conjugated (reference
        `tnkit/blocks.py:811-814`)."""
        return BT([l.flip() for l in self.legs], -self.charge,
                  {k: np.conj(b) for k, b in self.blocks.items()}, self.dtype)

    def scaled(self, c) -> "BT":
        return BT(self.legs, self.charge, {k: b * c for k, b in self.blocks.items()},
                  self.dtype)

    def norm(self) -> float:
        return float(np.sqrt(sum(float(np.vdot(b, b).real) for b in self.blocks.values())))

    def scale_leg(self, s: np.ndarray, axis: int) -> "BT":
        """Multiply leg `axis` by the vector `s` over its sector-ordered index (reference
        `tnkit/blocks.py:816-819`)."""
        starts = np.concatenate([[0], np.cumsum(self.legs[axis].dims)[:-1]]).astype(int)
        out = {}
        for k, b in self.blocks.items():
            sec = k[axis]
            v = s[starts[sec]:starts[sec] + self.legs[axis].dims[sec]]
            shp = [1] * b.ndim
            shp[axis] = -1
            out[k] = b * v.reshape(shp)
        return BT(self.legs, self.charge, out, self.dtype)


def tensordot(a: BT, b: BT, ax_a: Sequence[int], ax_b: Sequence[int]) -> BT:
    """Contract legs `ax_a` of `a` with legs `ax_b` of `b` block pair by block pair; the result
    has the free legs of `a`, then those of `b` (reference `tnkit/blocks.py:1156-1192`)."""
    ax_a, ax_b = tuple(ax_a), tuple(ax_b)
    for i, j in zip(ax_a, ax_b):
        la, lb = a.legs[i], b.legs[j]
        if la.charges != lb.charges or la.dims != lb.dims or la.sign != -lb.sign:
            raise ValueError(f"cannot contract leg {i} {la} with leg {j} {lb}")
    fa = [i for i in range(len(a.legs)) if i not in ax_a]
    fb = [j for j in range(len(b.legs)) if j not in ax_b]
    legs = [a.legs[i] for i in fa] + [b.legs[j] for j in fb]
    dtype = np.result_type(a.dtype, b.dtype)
    out = BT(legs, a.charge + b.charge, dtype=dtype)
    by_k: Dict[Tuple[int, ...], list] = {}
    for kb, blk in b.blocks.items():
        by_k.setdefault(tuple(kb[j] for j in ax_b), []).append((kb, blk))
    for ka, A in a.blocks.items():
        kc = tuple(ka[i] for i in ax_a)
        for kb, B in by_k.get(kc, ()):
            key = tuple(ka[i] for i in fa) + tuple(kb[j] for j in fb)
            out.blocks[key] = out.blocks[key] + np.tensordot(A, B, (ax_a, ax_b))
    return out


def einsum2(sub: str, a: BT, b: BT) -> BT:
    """A two-operand einsum without batch indices, as the reference's `BlockBackend.einsum`
    (`tnkit/block_backend.py:48-68`, `:121-131`): contract the shared letters, then permute."""
    lhs, outs = sub.replace(" ", "").split("->")
    ta, tb = lhs.split(",")
    shared = [c for c in ta if c in tb]
    t = tensordot(a, b, [ta.index(c) for c in shared], [tb.index(c) for c in shared])
    free = [c for c in ta if c not in shared] + [c for c in tb if c not in shared]
    perm = [free.index(c) for c in outs]
    return t if perm == list(range(len(perm))) else t.transpose(perm)


# --------------------------------------------------------------------------- #
# fuse / split of leg groups (reference `tnkit/blocks.py:1196-1286`)
# --------------------------------------------------------------------------- #
class FuseRec:
    """How groups of consecutive legs were fused: for each fused leg, its sectors (signed group
    totals, sorted) and, per fused sector, the stacked sub-sector tuples with offsets."""

    def __init__(self, legs, charge, groups):
        self.legs, self.charge, self.groups = tuple(legs), charge, groups
        self.fused, self.subs = [], []
        for g in groups:
            by_q: Dict[int, list] = {}
            for t in itertools.product(*(range(len(legs[a].charges)) for a in g)):
                q = sum(legs[a].sign * legs[a].charges[s] for a, s in zip(g, t))
                by_q.setdefault(q, []).append(t)
            qs = sorted(by_q)
            subs, dims = [], []
            for q in qs:
                off, items = 0, []
                for t in by_q[q]:
                    n = int(np.prod([legs[a].dims[s] for a, s in zip(g, t)]))
                    items.append((t, off, n))
                    off += n
                subs.append(items)
                dims.append(off)
            self.fused.append(Leg(tuple(qs), tuple(dims), 1))
            self.subs.append(subs)


def fuse(t: BT, groups) -> Tuple[BT, FuseRec]:
    """Fuse groups of consecutive legs (in order) into single legs of sign +1."""
    rec = FuseRec(t.legs, t.charge, [tuple(g) for g in groups])
    out = BT(rec.fused, t.charge, dtype=t.dtype)
    for key in out.keys:
        blk = out.blocks[key]
        for parts in itertools.product(*(rec.subs[g][key[g]] for g in range(len(groups)))):
            src = tuple(s for (tup, _, _) in parts for s in tup)
            sub = t.blocks.get(src)
            if sub is None:
                continue
            sl = tuple(slice(off, off + n) for (_, off, n) in parts)
            blk[sl] = sub.reshape(tuple(n for (_, _, n) in parts))
    return out, rec


def split(m: BT, rec: FuseRec, which: int) -> BT:
    """Split fused leg `which` of `m` (other legs kept) back into its group's legs."""
    g = rec.groups[which]
    legs = []
    for i, l in enumerate(m.legs):
        legs += [rec.legs[a] for a in g] if i == which else [l]
    out = BT(legs, m.charge, dtype=m.dtype)
    for key, blk in m.blocks.items():
        for (tup, off, n) in rec.subs[which][key[which]]:
            dims = [rec.legs[a].dims[s] for a, s in zip(g, tup)]
            sl = [slice(None)] * blk.ndim
            sl[which] = slice(off, off + n)
            piece = blk[tuple(sl)]
            shp = list(piece.shape[:which]) + dims + list(piece.shape[which + 1:])
            nk = key[:which] + tup + key[which + 1:]
            if nk in out.blocks:
                out.blocks[nk] = piece.reshape(shp).copy()
    return out


# --------------------------------------------------------------------------- #
# factorisations (reference `tnkit/blocks.py:1380-1495`)
# --------------------------------------------------------------------------- #
def _mat_blocks(m: BT):
    for k in m.keys:
        yield k[0], k[1], m.blocks[k]


def truncated_svd(m: BT, chi: int):
    """U, S, Vh, disc of a two-leg block tensor, keeping the `chi` largest singular values over
    all sectors (stable order of -sigma, then position), new bond sectors labelled by the row
    charge (reference `tnkit/blocks.py:1380-1462` with svd_tol = degenerate_tol = 0)."""
    lr, lc = m.legs
    parts = []
    for r, c, M in _mat_blocks(m):
        U, S, Vh = np.linalg.svd(M, full_matrices=False)
        parts.append((r, c, U, S, Vh))
    s_all = np.concatenate([p[3] for p in parts])
    owner = np.concatenate([np.full(len(p[3]), j) for j, p in enumerate(parts)])
    order = np.lexsort((np.arange(s_all.size), -s_all))
    k = min(chi, s_all.size)
    kept = np.bincount(owner[order[:k]], minlength=len(parts))
    disc = float(np.sum(s_all[order[k:]] ** 2))
    new = []
    for (r, c, U, S, Vh), n in zip(parts, kept.tolist()):
        if n:
            lab = lr.charges[r] if lr.sign > 0 else -lr.charges[r]
            new.append((lab, r, c, U[:, :n], S[:n], Vh[:n]))
    new.sort(key=lambda x: (x[0], x[1]))
    bond = Leg(tuple(x[0] for x in new), tuple(len(x[4]) for x in new), 1)
    Ut = BT([lr, bond.flip()], 0, dtype=m.dtype)
    Vt = BT([bond, lc], m.charge, dtype=m.dtype)
    for j, (lab, r, c, U, S, Vh) in enumerate(new):
        Ut.blocks[(r, j)] = U
        Vt.blocks[(j, c)] = Vh
    S = np.concatenate([x[4] for x in new])
    return Ut, S, Vt, disc


def qr_right(m: BT):
    """m = L Q block by block with Q having orthonormal rows (reference `tnkit/blocks.py:1465-
    1495`, right=True): per block q, t = qr(M^H), L = t^H, Q = q^H."""
    lr, lc = m.legs
    new = []
    for r, c, M in _mat_blocks(m):
        q, t = np.linalg.qr(M.conj().T)
        lab = lr.charges[r] if lr.sign > 0 else -lr.charges[r]
        new.append((lab, r, c, t.conj().T, q.conj().T))
    new.sort(key=lambda x: x[0])
    bond = Leg(tuple(x[0] for x in new), tuple(int(x[3].shape[1]) for x in new), 1)
    A = BT([lr, bond.flip()], 0, dtype=m.dtype)
    B = BT([bond, lc], m.charge, dtype=m.dtype)
    for j, (lab, r, c, a, b) in enumerate(new):
        A.blocks[(r, j)] = a
        B.blocks[(j, c)] = b
    return A, B
