"""Oracle restatement of the DMRG inner loop (numpy, CPU; test infrastructure only).

Functions follow the reference tnkit 0.3.0 one for one:
  apply_two_site        tnkit/_dmrg.py:162-169   (block or dense operands)
  fused_two_site        tnkit/_dmrg.py:172-180   (dense)
  apply_two_site_fused  tnkit/_dmrg.py:183-189   (dense)
  apply_one_site        tnkit/_dmrg.py:192-199
  update_left_env       tnkit/_dmrg.py:216-222
  update_right_env      tnkit/_dmrg.py:225-231
  edge_envs             tnkit/_dmrg.py:234-247
  lanczos_ground_restart tnkit/eigensolver.py:507-674
  mpo_charges / to_block_mpo  tnkit/block_backend.py:162-256
  random_block_mps      tnkit/block_backend.py:259-311
  right_canonicalize    tnkit/_dmrg.py:295-306 (blocks, per-block LQ)
  dmrg                  tnkit/_dmrg.py:560-799 (two-site, trunc='svd', expand=0)
"""
from __future__ import annotations

import time
from typing import List, Sequence

import numpy as np

from .blocks_np import BT, Leg, einsum2, fuse, qr_right, split, truncated_svd


def _es(sub, a, b):
    if isinstance(a, BT):
        return einsum2(sub, a, b)
    return np.einsum(sub, a, b, optimize=True)


def _conj(x):
    return x.conj() if isinstance(x, BT) else np.conj(x)


# --------------------------------------------------------------------------- #
# local contractions
# --------------------------------------------------------------------------- #
def apply_two_site(theta, L, W1, W2, R):
    """out[p,s,t,d] = sum L[p,w,q] th[q,i,j,b] W1[w,m,s,i] W2[m,r,t,j] R[d,r,b] as the
    reference's four pairwise contractions (tnkit/_dmrg.py:165-168)."""
    x1 = _es("pwq,qijb->pwijb", L, theta)
    x2 = _es("wmsi,pwijb->pmsjb", W1, x1)
    x3 = _es("mrtj,pmsjb->pstrb", W2, x2)
    return _es("drb,pstrb->pstd", R, x3)


def fused_two_site(L, W1, W2, R):
    """Dense: L as (p*wl, q), the MPO pair as S[(s t wr), (wl i j)], R as (d, wr*b)."""
    p, wl, q = L.shape
    wr, d1, d2 = W2.shape[1], W1.shape[2], W2.shape[2]
    S = np.einsum("wmsi,mrtj->strwij", W1, W2).reshape(d1 * d2 * wr, wl * d1 * d2)
    return L.reshape(p * wl, q), S, R.reshape(R.shape[0], wr * R.shape[2])


def apply_two_site_fused(theta, Lm, S, Rm):
    q, d1, d2, b = theta.shape
    x = (Lm @ theta.reshape(q, -1)).reshape(-1, S.shape[1], b)
    x = S @ x
    return (x.reshape(-1, Rm.shape[1]) @ Rm.T).reshape(-1, d1, d2, Rm.shape[0])


def apply_one_site(M, L, W, R):
    x1 = _es("aky,ysb->aksb", L, M)
    x2 = _es("klst,aktb->alsb", W, x1)
    return _es("bly,alsy->asb", R, x2)


def update_left_env(L, A, W):
    t1 = _es("pwq,psd->wqsd", L, _conj(A))
    t2 = _es("wqsd,wrsy->qdry", t1, W)
    return _es("qdry,qye->dre", t2, A)


def update_right_env(R, B, W):
    t1 = _es("xry,usx->ryus", R, _conj(B))
    t2 = _es("ryus,wrsp->yuwp", t1, W)
    return _es("yuwp,vpy->uwv", t2, B)


def two_site_macs(theta: BT, L: BT, W1: BT, W2: BT, R: BT) -> int:
    """Multiply-adds of the four block contractions of `apply_two_site`: the reference's
    algorithmic count, sum over block pairs of the GEMM sizes (tnkit/blocks.py:1089-1090 sums
    R*K*C per charge group; summed over block pairs it is the same number)."""
    def macs(a, b, ax_a, ax_b):
        n = 0
        by = {}
        for kb in b.keys:
            by.setdefault(tuple(kb[j] for j in ax_b), []).append(kb)
        for ka in a.keys:
            kc = tuple(ka[i] for i in ax_a)
            sa = a.shape_of(ka)
            for kb in by.get(kc, ()):
                sb = b.shape_of(kb)
                n += int(np.prod(sa)) * int(np.prod([sb[j] for j in range(len(sb))
                                                     if j not in ax_b]))
        return n
    tot = macs(L, theta, (2,), (0,))
    x1 = einsum2("pwq,qijb->pwijb", L, theta)
    tot += macs(W1, x1, (0, 3), (1, 2))
    x2 = einsum2("wmsi,pwijb->pmsjb", W1, x1)
    tot += macs(W2, x2, (0, 3), (1, 3))
    x3 = einsum2("mrtj,pmsjb->pstrb", W2, x2)
    tot += macs(R, x3, (1, 2), (3, 4))
    return tot


# --------------------------------------------------------------------------- #
# block MPO / MPS construction
# --------------------------------------------------------------------------- #
def leg_from_charges(q, sign=1):
    """(Leg, stable order of the dense indices by sector) (tnkit/blocks.py:103-118, U(1))."""
    q = np.asarray(q, dtype=np.int64)
    c, n = np.unique(q, return_counts=True)
    return Leg(tuple(int(x) for x in c), tuple(int(x) for x in n), sign), np.argsort(q,
                                                                               kind="stable")


def from_dense(x, legs, charge=0, orders=None) -> BT:
    for i, o in enumerate(orders or ()):
        if o is not None:
            x = np.take(x, o, axis=i)
    t = BT(legs, charge, dtype=np.asarray(x).dtype)
    starts = [np.concatenate([[0], np.cumsum(l.dims)[:-1]]).astype(int) for l in legs]
    for k in t.keys:
        sl = tuple(slice(starts[i][s], starts[i][s] + legs[i].dims[s]) for i, s in enumerate(k))
        t.blocks[k] = np.array(x[sl])
    return t


def mpo_charges(mpo, site_charges, tol=0.0):
    """Charge of every MPO channel (tnkit/block_backend.py:162-208, U(1), left = trivial)."""
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
        found = {int(j): set() for j in np.flatnonzero(live[n + 1])}
        for i, j, x, y in zip(a, b, s, t):
            if live[n][i] and live[n + 1][j]:
                found[int(j)].add(int(out[-1][i] + q[x] - q[y]))
        qr = np.zeros(W.shape[1], np.int64)
        for j, vals in found.items():
            if len(vals) != 1:
                raise ValueError(f"MPO site {n}, channel {j}: charges {sorted(vals)}")
            qr[j] = vals.pop()
        out.append(qr)
    return out


def to_block_mpo(mpo, site_charges, tol=0.0):
    """Dense MPO -> block tensors with legs (wl, wr, s, s') of signs (+1, -1, +1, -1)
    (tnkit/block_backend.py:211-256)."""
    chans = mpo_charges(mpo, site_charges, tol)
    out = []
    for n, W in enumerate(mpo):
        cl, ol = leg_from_charges(chans[n])
        cr, orr = leg_from_charges(chans[n + 1])
        p, op = leg_from_charges(site_charges[n])
        out.append(from_dense(np.asarray(W, dtype=np.float64), (cl, cr.flip(), p, p.flip()), 0,
                              (ol, orr, op, op)))
    return out


def random_block_mps(mpo: Sequence[BT], chi: int, charge: int, rng) -> List[BT]:
    """Random block MPS of total charge `charge` (tnkit/block_backend.py:259-311)."""
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
    legs = []
    for b in bonds:
        cs = sorted(b)
        legs.append(Leg(tuple(cs), tuple(b[c] for c in cs), 1))
    out = []
    for n, p in enumerate(phys):
        t = BT((legs[n], p, legs[n + 1].flip()), 0)
        out.append(BT.from_flat(t.legs, 0, rng.standard_normal((t.size,))))
    return out


def right_canonicalize(M: List[BT]) -> List[BT]:
    """Per-block LQ from the right, centre renormalised at every step (tnkit/_dmrg.py:295-306)."""
    for i in range(len(M) - 1, 0, -1):
        f, rec = fuse(M[i], ((0,), (1, 2)))
        Lm, Q = qr_right(f)
        M[i] = split(Q, rec, 1)
        Lm = split(Lm, rec, 0)
        M[i - 1] = einsum2("asb,bc->asc", M[i - 1], Lm)
        M[i - 1] = M[i - 1].scaled(1.0 / M[i - 1].norm())
    M[0] = M[0].scaled(1.0 / M[0].norm())
    return M


def edge_envs(M: List[BT], mpo: List[BT]):
    a, b = M[0].legs[0], M[-1].legs[2]
    one = np.ones((1, 1, 1))
    return (from_dense(one, (a, mpo[0].legs[0].flip(), a.flip())),
            from_dense(one, (b, mpo[-1].legs[1].flip(), b.flip())))


# --------------------------------------------------------------------------- #
# thick-restart Lanczos (tnkit/eigensolver.py:507-674), reorth 'cgs2'
# --------------------------------------------------------------------------- #
def lanczos_ground_restart(matvec, v0, tol=1e-8, max_iter=200, m=40, k=10):
    if k >= m:
        k = max(1, m // 2)
    n0 = float(np.linalg.norm(v0))
    if not np.isfinite(n0) or n0 < 1e-300:
        return 0.0, v0, {"iters": 0, "converged": False, "restarts": 0}
    n = v0.size
    Vb = np.zeros((m + 1, n), dtype=v0.dtype)
    Vb[0] = v0.reshape(-1) / n0
    nV = 1
    T = np.zeros((m + 1, m + 1))
    n_kept, border = 0, None
    beta_prev, v_prev = 0.0, np.zeros(n, dtype=v0.dtype)
    theta, y = 0.0, np.array([1.0])
    converged, restarts, it, j = False, 0, 0, 0
    while it < max_iter:
        v = Vb[j]
        w = matvec(v)
        if n_kept and j == n_kept:
            w = w - border @ Vb[:n_kept]
        elif j > 0:
            w = w - beta_prev * v_prev
        alpha = float(np.vdot(v, w).real)
        w = w - alpha * v
        Vl = Vb[:nV]
        for _ in range(2):
            c = np.conj(Vl) @ w
            w = w - c @ Vl
        T[j, j] = alpha
        beta = float(np.linalg.norm(w))
        cur = j + 1
        if cur == 1:
            th, y = alpha, np.array([1.0])
        else:
            ev, evec = np.linalg.eigh(T[:cur, :cur])
            th, y = float(ev[0]), evec[:, 0]
        it += 1
        res = abs(beta) * abs(float(y[-1]))
        breakdown = (not np.isfinite(beta) or not np.isfinite(alpha)
                     or beta < 1e-12 * max(1.0, abs(alpha)))
        theta = th
        if breakdown or res < tol:
            converged = True
            break
        if cur >= m:
            ev, evec = np.linalg.eigh(T[:cur, :cur])
            kk = min(k, cur - 1)
            Yk = evec[:, :kk]
            vnew = w / beta
            Vb[:kk] = Yk.T @ Vb[:cur]
            Vb[kk] = vnew
            nV = kk + 1
            T[:] = 0.0
            border = beta * Yk[cur - 1, :]
            for i in range(kk):
                T[i, i] = ev[i]
                T[i, kk] = T[kk, i] = border[i]
            n_kept, j = kk, kk
            beta_prev, v_prev = 0.0, np.zeros(n, dtype=v0.dtype)
            y = np.zeros(kk + 1)
            y[0] = 1.0
            restarts += 1
            continue
        T[j, j + 1] = T[j + 1, j] = beta
        v_prev, beta_prev = v, beta
        Vb[j + 1] = w / beta
        nV = j + 2
        j += 1
    ny = min(len(y), nV)
    x = y[:ny] @ Vb[:ny]
    x = x / np.linalg.norm(x)
    return theta, x, {"iters": it, "converged": converged, "restarts": restarts}


# --------------------------------------------------------------------------- #
# two-site block DMRG (tnkit/_dmrg.py:560-799, trunc='svd', expand=0, warm start)
# --------------------------------------------------------------------------- #
def dmrg_blocks(mpo: List[BT], chi: int, charge: int = 0, n_sweeps: int = 4, seed: int = 0,
                eig_tol: float = 1e-9, m: int = 40, k: int = 10, init=None):
    N = len(mpo)
    M = (list(init) if init is not None
         else random_block_mps(mpo, chi, charge, np.random.default_rng(seed)))
    M = right_canonicalize(M)
    L = [None] * (N + 1)
    R = [None] * (N + 1)
    L[0], R[N] = edge_envs(M, mpo)
    for i in range(N - 1, 0, -1):
        R[i] = update_right_env(R[i + 1], M[i], mpo[i])
    energies, sweep_s, total_disc, mv = [], [], 0.0, [0]

    def solve(i, right):
        nonlocal total_disc
        th0 = einsum2("asc,ctb->astb", M[i], M[i + 1])
        legs, q = th0.legs, th0.charge

        def matvec(x):
            mv[0] += 1
            return apply_two_site(BT.from_flat(legs, q, x), L[i], mpo[i], mpo[i + 1],
                                  R[i + 2]).flat()
        mi = min(th0.size, max(200, 4 * chi))
        e, x, _ = lanczos_ground_restart(matvec, th0.flat(), tol=eig_tol, max_iter=mi, m=m, k=k)
        mat, rec = fuse(BT.from_flat(legs, q, x), ((0, 1), (2, 3)))
        U, S, Vh, disc = truncated_svd(mat, chi)
        S = S / np.linalg.norm(S)
        if right:
            M[i] = split(U, rec, 0)
            M[i + 1] = split(Vh.scale_leg(S, 0), rec, 1)
            L[i + 1] = update_left_env(L[i], M[i], mpo[i])
        else:
            M[i] = split(U.scale_leg(S, 1), rec, 0)
            M[i + 1] = split(Vh, rec, 1)
            R[i + 1] = update_right_env(R[i + 2], M[i + 1], mpo[i + 1])
        total_disc += disc
        return e

    E = None
    for _ in range(n_sweeps):
        t0 = time.perf_counter()
        for i in range(N - 1):
            E = solve(i, True)
        for i in range(N - 2, -1, -1):
            E = solve(i, False)
        energies.append(E)
        sweep_s.append(time.perf_counter() - t0)
    return E, M, {"energies": energies, "sweep_s": sweep_s, "discarded_weight": total_disc,
                  "matvec_calls": mv[0]}


def dense_as_blocks(W: Sequence[np.ndarray]) -> List[BT]:
    """A dense MPO as single-sector (trivial charge) block tensors, so the dense problem runs
    through the same sweep."""
    out = []
    for w in W:
        wl, wr, d, _ = w.shape
        legs = (Leg((0,), (wl,), 1), Leg((0,), (wr,), -1), Leg((0,), (d,), 1),
                Leg((0,), (d,), -1))
        out.append(BT(legs, 0, {(0, 0, 0, 0): np.asarray(w, dtype=np.float64)}))
    return out


def random_dense_mps(N, chi, d, rng) -> List[BT]:
    """Dense random MPS as single-sector blocks, drawn as the reference's `random_mps`
    (tnkit/_dmrg.py:253-261)."""
    dims = [1] + [min(chi, d ** min(i, N - i)) for i in range(1, N)] + [1]
    out = []
    for i in range(N):
        x = rng.standard_normal((dims[i], d, dims[i + 1]))
        legs = (Leg((0,), (dims[i],), 1), Leg((0,), (d,), 1), Leg((0,), (dims[i + 1],), -1))
        out.append(BT(legs, 0, {(0, 0, 0): x}))
    return out
