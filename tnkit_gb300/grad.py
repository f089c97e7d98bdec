"""Gradients through the hot-path kernels.

  TwoSiteMatvec      torch.autograd.Function: y = H_eff theta on the tnk kernels; its backward
                     g_theta = H_eff^T g_y is the same two-site contraction on the transposed
                     operator (environments with every leg reversed and flipped, by one
                     tnk_combine_f64 launch each; MPO tensors with their physical legs swapped
                     and channel legs flipped), so the gradient of any scalar of y reaches theta
                     -- for the local energy theta^T H_eff theta, 2 H_eff theta for a symmetric
                     H_eff
  bond_expectations  <psi| h_{i,i+1} |psi> for every bond of an MPS: the two-site operator h
                     applied by the same matvec kernel with identity environments at the bond's
                     orthogonality centre, the centre moved left to right by exact SVD steps.
                     For H(J) = sum_i J_i h_i these are the Hellmann-Feynman derivatives
                     dE/dJ_i = <psi| dH/dJ_i |psi> at a ground state
  energy_gradient_xxz  dE/dJ_i of the disordered XXZ chain from a DMRG ground state
  tdvp_observable_gradient  <Z_j(t)> after two-site TDVP and d<Z_j(t)>/dJ_i for every bond, by
                     the continuous adjoint: psi(s) forward and lam(s) = exp(iH(t-s)) Z psi(t)
                     backward by tdvp2_evolve, Im <lam(s)|h_i|psi(s)> at every step from two
                     same-state bond values of the MPS sums lam -+ i psi (mps_sum: direct-sum
                     bonds, built by block copies on the device; bond_values: identity-MPO
                     environments and the matvec kernel, any gauge), integrated by Boole's rule

The reference has no gradients: the oracles are central finite differences of its energies and
Hellmann-Feynman expectation values (the bond operator's MPO, as tnkit/dmrg_excited.py:185-211
measures one); the tests also check against exact diagonalisation and torch's numerical
Jacobian.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np
import torch

from . import linalg as LA
from . import ops
from . import plan as P
from .layout import canonical, from_dense_np, to_dense_np
from .mpo import to_block_mpo
from .tensor import BlockTensor

# --------------------------------------------------------------------------------------------
# transposed operators
# --------------------------------------------------------------------------------------------


def _plan_reverse3(lay) -> P.HostCombPlan:
    """Combination plan of T[a, w, b] -> T'[b, w, a] (3 legs reversed, every sign flipped):
    one strided 2-D copy per block and middle index."""
    a, w, b = lay.legs
    out = canonical((b.flip(), w.flip(), a.flip()), _neg(lay.charge))
    c = P.CombTable()
    for k in range(lay.nblocks):
        ka, kw, kb = lay.key(k)
        A, Wd, B = lay.shape(k)
        ko = out.index[(kb, kw, ka)]
        so, do = int(lay.offsets[k]), int(out.offsets[ko])
        for j in range(Wd):
            # dst[q, j, p] (row q, column p) from src[p, j, q]
            c.add(do + j * A, B, A, Wd * A, 1, [P.term(so + j * B, 1, Wd * B, 1.0)])
    return P.HostCombPlan(c, out)


def _neg(q):
    return tuple(-x for x in q) if isinstance(q, tuple) else -q


def transpose_env(E: BlockTensor) -> BlockTensor:
    """An environment (a, w, b) as its transpose (b, w, a) with every leg flipped: the operator
    of the adjoint contraction. One tnk_combine_f64 launch."""
    p = ops._PLANS.get_or(("rev3", E.layout, str(E.data.device)),
                          lambda: ops.DeviceCombPlan(_plan_reverse3(E.layout), E.data.device))
    out = torch.empty(p.out_layout.size, dtype=E.data.dtype, device=E.data.device)
    p.run(E.data, out)
    return BlockTensor(p.out_layout, out)


def transpose_mpo(W: BlockTensor) -> BlockTensor:
    """W[wl, wr, s, s'] -> W^T[wl, wr, s', s] with the channel legs flipped (host side: MPO
    tensors are a few hundred numbers)."""
    wl, wr, s, sp = W.layout.legs
    dense = to_dense_np(W.layout, ops._host_of(W))
    lay = canonical((wl.flip(), wr.flip(), sp.flip(), s.flip()), _neg(W.layout.charge))
    host = from_dense_np(lay, np.ascontiguousarray(dense.transpose(0, 1, 3, 2)))
    return BlockTensor(lay, torch.as_tensor(host, device=W.data.device), host)


class TwoSiteMatvec(torch.autograd.Function):
    """y = H_eff(L, W1, W2, R) theta with the gradient of theta: forward and backward are both
    the two-site grouped-GEMM kernels (the backward on the transposed operator). L, R, W1, W2
    are constants of the local problem (BlockTensors); theta is the flat FP64 CUDA buffer."""

    @staticmethod
    def forward(ctx, theta, layout, L, W1, W2, R):
        op = ops.TwoSiteOperator(layout, L, W1, W2, R)
        ctx.problem = (layout, L, W1, W2, R)
        return op(theta.detach().contiguous())

    @staticmethod
    def backward(ctx, gy):
        layout, L, W1, W2, R = ctx.problem
        opT = ops.TwoSiteOperator(layout, transpose_env(L), transpose_mpo(W1),
                                  transpose_mpo(W2), transpose_env(R))
        return opT(gy.contiguous()), None, None, None, None, None


def local_energy(theta, layout, L, W1, W2, R):
    """theta^T H_eff theta / theta^T theta as a differentiable function of theta."""
    y = TwoSiteMatvec.apply(theta, layout, L, W1, W2, R)
    return torch.dot(theta, y) / torch.dot(theta, theta)


# --------------------------------------------------------------------------------------------
# Hellmann-Feynman: bond expectation values
# --------------------------------------------------------------------------------------------


def xxz_bond_operator(delta: float = 1.0) -> List[np.ndarray]:
    """The two-site MPO (1,3,2,2), (3,1,2,2) of h = (S+S- + S-S+)/2 + delta Sz Sz."""
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm, sz = sp.T.copy(), np.diag([0.5, -0.5])
    W1 = np.zeros((1, 3, 2, 2))
    W2 = np.zeros((3, 1, 2, 2))
    W1[0, 0], W1[0, 1], W1[0, 2] = sp, sm, sz
    W2[0, 0], W2[1, 0], W2[2, 0] = 0.5 * sm, 0.5 * sp, delta * sz
    return [W1, W2]


def _identity_env(outer, middle, device):
    """Identity environment with legs (outer, middle, outer.flip()) and one channel on the
    middle leg: blocks (q, 0, q) are identity matrices."""
    lay = canonical((outer, middle, outer.flip()),
                    tuple(0 for _ in outer.charges[0]) if isinstance(outer.charges[0], tuple)
                    else 0)
    host = np.zeros(lay.size)
    for k in range(lay.nblocks):
        a, _, b = lay.shape(k)
        if lay.key(k)[0] == lay.key(k)[2]:
            o = int(lay.offsets[k])
            host[o:o + a * b].reshape(a, b)[np.diag_indices(a)] = 1.0
    return BlockTensor(lay, torch.as_tensor(host, device=device), host)


def bond_expectations(mps: Sequence[BlockTensor], bond_op: Sequence[BlockTensor]) -> np.ndarray:
    """<psi| h_{i,i+1} |psi> / <psi|psi> for i = 0 .. N-2, with h given as a two-site block MPO
    (channel legs trivial at both ends). `mps` must have its orthogonality centre on site 0 and
    sites 1.. right-canonical, as `dmrg` returns it; it is not modified."""
    M = [BlockTensor(m.layout, m.data.clone()) for m in mps]
    W1, W2 = bond_op
    N = len(M)
    out = np.zeros(N - 1)
    for i in range(N - 1):
        theta = ops.tensordot(M[i], M[i + 1], 1)
        # the environments a two-site contraction expects: L (a, wl.flip(), a.flip()) and
        # R (b, wr.flip(), b.flip()) for theta's outer legs a, b
        L = _identity_env(theta.legs[0], W1.legs[0].flip(), theta.data.device)
        R = _identity_env(theta.legs[3], W2.legs[1].flip(), theta.data.device)
        y = ops.apply_two_site(theta, L, W1, W2, R)
        nn = float(torch.dot(theta.data, theta.data))
        out[i] = float(torch.dot(theta.data, y.data)) / nn
        if i < N - 2:
            mat, info = LA.fuse_matrix(theta, 2)
            keep = int(sum(mat.layout.legs[0].dims))
            U, S, Vh, _ = LA.truncated_svd(mat, keep, scale="right", normalize=False,
                                           driver="gesvd")
            M[i] = LA.split_rows(U, info)
            M[i + 1] = LA.split_cols(Vh, info)
    return out


def energy_gradient_xxz(mps: Sequence[BlockTensor], delta: float = 1.0) -> np.ndarray:
    """dE/dJ_i of H = sum_i J_i [(S+S- + S-S+)/2 + delta Sz Sz]_{i,i+1} at the DMRG state `mps`
    (Hellmann-Feynman: the bond expectation values)."""
    dev = mps[0].data.device
    Wb, _ = to_block_mpo(xxz_bond_operator(delta), [[1, -1]] * 2, device=dev)
    return bond_expectations(mps, Wb)


# --------------------------------------------------------------------------------------------
# gradients with respect to the MPS tensors, by environment recomputation
# --------------------------------------------------------------------------------------------


def _identity_mpo(W: Sequence[BlockTensor]) -> List[BlockTensor]:
    """The identity MPO with the physical legs of `W` (channel legs one-dimensional)."""
    dense = [np.eye(w.legs[2].size)[None, None] for w in W]
    if all(len(w.legs[2].charges) == 1 for w in W) and all(len(w.legs[0].charges) == 1
                                                           for w in W):
        from .mpo import dense_mpo
        return dense_mpo(dense, device=W[0].data.device)
    labels = [[c for c, d in zip(w.legs[2].charges, w.legs[2].dims) for _ in range(d)]
              for w in W]
    return to_block_mpo(dense, labels, device=W[0].data.device)[0]


def _network(M, W):
    """All left environments L[0..N] and right environments R[0..N] of <psi|W|psi>."""
    from .dmrg import edge_envs
    N = len(M)
    dev = M[0].data.device
    L: list = [None] * (N + 1)
    R: list = [None] * (N + 1)
    L[0], R[N] = edge_envs(M, W, dev)
    for i in range(N):
        L[i + 1] = ops.update_left_env(L[i], M[i], W[i])
    for i in range(N - 1, -1, -1):
        R[i] = ops.update_right_env(R[i + 1], M[i], W[i])
    return L, R


def mps_energy_gradient(mps: Sequence[BlockTensor], mpo: Sequence[BlockTensor]):
    """E = <psi|H|psi> / <psi|psi> of a real MPS and dE/dA_i for every site tensor, by
    environment recomputation: the derivative of the network <psi|H|psi> with respect to A_i
    is the network with A_i taken out, i.e. 2 H_eff^(i) A_i -- the one-site effective operator
    (L_i, W_i, R_i+1) applied to A_i by the one-site matvec kernel -- and likewise for the norm
    with the identity MPO; dE/dA_i = (2 H_eff A_i - 2 E N_eff A_i) / <psi|psi>. No canonical
    form is assumed. Returns (E, [dE/dA_i as BlockTensors with the layouts of the A_i])."""
    M = list(mps)
    W = list(mpo)
    if any(m.data.is_complex() for m in M):
        raise TypeError("mps_energy_gradient takes a real MPS")
    Wn = _identity_mpo(W)
    Lh, Rh = _network(M, W)
    Ln, Rn = _network(M, Wn)
    f = float(Lh[len(M)].data.sum())
    nrm = float(Ln[len(M)].data.sum())
    E = f / nrm
    grads = []
    for i, A in enumerate(M):
        h = ops.apply_one_site(A, Lh[i], W[i], Rh[i + 1]).data
        n = ops.apply_one_site(A, Ln[i], Wn[i], Rn[i + 1]).data
        grads.append(BlockTensor(A.layout, (2.0 / nrm) * (h - E * n)))
    return E, grads


# --------------------------------------------------------------------------------------------
# gradient of a time-evolved observable: two-site TDVP and its continuous adjoint
# --------------------------------------------------------------------------------------------


def clone_mps(mps: Sequence[BlockTensor]) -> List[BlockTensor]:
    return [BlockTensor(m.layout, m.data.clone()) for m in mps]


def apply_pauli_z(mps: Sequence[BlockTensor], site: int) -> List[BlockTensor]:
    """Z_site |psi> on a U(1) S^z chain (physical charges 2 S^z = +-1): Z = 2 S^z is +1 on the
    blocks of charge +1 and -1 on those of charge -1 of the site tensor; a copy."""
    out = clone_mps(mps)
    A = out[site]
    lay = A.layout
    phys = lay.legs[1]
    for k in range(lay.nblocks):
        q = phys.charges[lay.key(k)[1]]
        if isinstance(q, tuple) or q not in (1, -1):
            raise ValueError("apply_pauli_z needs a spin-1/2 S^z chain (physical charges +-1)")
        if q < 0:
            o = int(lay.offsets[k])
            A.data[o:o + int(lay.sizes[k])].neg_()
    return out


def _leg_sum(a, b):
    """The direct sum of two bond legs of one sign: per charge the dims add."""
    from .layout import Leg
    if a.sign != b.sign:
        raise ValueError("bond legs of different signs")
    da = dict(zip(a.charges, a.dims))
    db = dict(zip(b.charges, b.dims))
    ch = tuple(sorted(set(da) | set(db)))
    return Leg(ch, tuple(da.get(c, 0) + db.get(c, 0) for c in ch), a.sign)


def mps_sum(a: Sequence[BlockTensor], b: Sequence[BlockTensor], cb: complex) -> List[BlockTensor]:
    """The MPS of |a> + cb |b>: every inner bond the direct sum of the two states' bonds, the
    site tensors block-diagonal in them (b's states after a's within each charge sector), the
    first site [A | cb B] and the last [A ; B] along their one open bond. Both MPS have the
    leg order (left bond, physical, right bond) of `random_block_mps`, the same physical legs
    and the same outer bonds. Built on the device by block copies."""
    from .layout import layout_of
    N = len(a)
    if N != len(b) or N < 1:
        raise ValueError("mps_sum needs two MPS of the same length")
    dev = a[0].data.device
    out = []
    for n in range(N):
        A, B = a[n], b[n]
        la, pa, ra = A.legs
        lb, pb, rb = B.legs
        if pa != pb or A.layout.charge != B.layout.charge:
            raise ValueError(f"site {n}: physical legs or charges differ")
        first, last = n == 0, n == N - 1
        if (first and la != lb) or (last and ra != rb):
            raise ValueError("the two MPS have different outer bonds")
        left = la if first else _leg_sum(la, lb)
        right = ra if last else _leg_sum(ra, rb)
        lay = layout_of((left, pa, right), A.layout.charge)
        data = torch.zeros(lay.size, dtype=torch.complex128, device=dev)
        dla, dra = dict(zip(la.charges, la.dims)), dict(zip(ra.charges, ra.dims))
        for T, coef, is_b in ((A, 1.0, False), (B, cb if first else 1.0, True)):
            tl = T.layout
            for k in range(tl.nblocks):
                il, ip, ir = tl.key(k)
                ql, qr = T.legs[0].charges[il], T.legs[2].charges[ir]
                kk = lay.index[(left.charges.index(ql), ip, right.charges.index(qr))]
                sl, sp, sr = tl.shape(k)
                lo = dla.get(ql, 0) if (is_b and not first) else 0
                ro = dra.get(qr, 0) if (is_b and not last) else 0
                o, oo = int(tl.offsets[k]), int(lay.offsets[kk])
                dst = data[oo:oo + int(lay.sizes[kk])].view(lay.shape(kk))
                src = T.data[o:o + sl * sp * sr].view(sl, sp, sr)
                dst[lo:lo + sl, :, ro:ro + sr] += coef * src
        out.append(BlockTensor(lay, data))
    return out


def _complex_envs(M: Sequence[BlockTensor], W: Sequence[BlockTensor]):
    """All left (L[0..N]) and right (R[0..N]) environments of <M|W|M> for a complex MPS in any
    gauge."""
    from .dmrg import edge_envs
    N = len(M)
    dev = M[0].data.device
    L: list = [None] * (N + 1)
    R: list = [None] * (N + 1)
    L0, RN = edge_envs(M, W, dev)
    L[0] = BlockTensor(L0.layout, L0.data.to(torch.complex128))
    R[N] = BlockTensor(RN.layout, RN.data.to(torch.complex128))
    for i in range(N):
        L[i + 1] = ops.update_left_env(L[i], M[i], W[i])
    for i in range(N - 1, -1, -1):
        R[i] = ops.update_right_env(R[i + 1], M[i], W[i])
    return L, R


def bond_values(M: Sequence[BlockTensor], W_id: Sequence[BlockTensor],
                bond_op: Sequence[BlockTensor]) -> np.ndarray:
    """<M| h_{i,i+1} |M> for every bond i, unnormalised and in any gauge: the identity-MPO
    environments left of i and right of i+1, and the two-site operator h applied to the bond's
    two site tensors by the matvec kernel (W_id: the identity MPO of the chain, whose channel
    legs are those of h's outer channels)."""
    M = list(M)
    N = len(M)
    L, R = _complex_envs(M, W_id)
    W1, W2 = bond_op
    out = np.zeros(N - 1)
    for i in range(N - 1):
        th = ops.tensordot(M[i], M[i + 1], 1)
        y = ops.apply_two_site(th, L[i], W1, W2, R[i + 2])
        out[i] = float(torch.vdot(th.data, y.data).real)
    return out


def im_transition_values(lam: Sequence[BlockTensor], psi: Sequence[BlockTensor],
                         W_id: Sequence[BlockTensor], bond_op: Sequence[BlockTensor]) -> np.ndarray:
    """Im <lam| h_i |psi> for every bond, by polarisation over two sums of the states: with
    A = <lam|h|lam> and B = <psi|h|psi>, <lam -+ i psi| h |lam -+ i psi> = A + B +- 2 Im <lam|h|psi>."""
    m = bond_values(mps_sum(lam, psi, -1j), W_id, bond_op)
    p = bond_values(mps_sum(lam, psi, 1j), W_id, bond_op)
    return (m - p) / 4.0


def quadrature_weights(n: int, dt: float) -> np.ndarray:
    """Weights of a composite closed Newton-Cotes rule on n + 1 equidistant points: Boole's
    rule when 4 divides n, Simpson's when 2 does, else Simpson's with the 3/8 rule on the last
    three intervals (trapezoid for n = 1)."""
    if n < 1:
        raise ValueError("a quadrature needs at least one interval")
    w = np.zeros(n + 1)
    if n == 1:
        w[:] = dt / 2
    elif n % 4 == 0:
        for a in range(0, n, 4):
            w[a:a + 5] += np.array([7.0, 32.0, 12.0, 32.0, 7.0]) * (2.0 * dt / 45.0)
    else:
        m = n if n % 2 == 0 else n - 3
        for a in range(0, m, 2):
            w[a:a + 3] += np.array([1.0, 4.0, 1.0]) * (dt / 3.0)
        if m < n:
            w[m:m + 4] += np.array([1.0, 3.0, 3.0, 1.0]) * (3.0 * dt / 8.0)
    return w


_AUX_MPOS: dict = {}


def _aux_mpo(kind: str, W: Sequence[BlockTensor], site: int = -1) -> List[BlockTensor]:
    """The identity MPO (kind 'id') or the Pauli Z MPO on `site` (kind 'z') of the chain of `W`,
    one object per (kind, physical legs, site, device): the matvec and environment plans are
    cached by MPO object, so repeated evaluations reuse them."""
    key = (kind, tuple(w.legs[2] for w in W), site, str(W[0].data.device))
    got = _AUX_MPOS.get(key)
    if got is None:
        got = _AUX_MPOS[key] = _identity_mpo(W) if kind == "id" else _z_mpo(W, site)
    return got


def _z_mpo(W: Sequence[BlockTensor], site: int) -> List[BlockTensor]:
    """The MPO of Pauli Z on `site` (identity elsewhere) with the physical legs of `W`."""
    dense = []
    for n, w in enumerate(W):
        d = w.legs[2].size
        dense.append(np.eye(d)[None, None] if n != site else np.diag([1.0, -1.0])[None, None])
    return to_block_mpo(dense, [[1, -1]] * len(W), device=W[0].data.device)[0]


def z_expectation(mps: Sequence[BlockTensor], mpo: Sequence[BlockTensor], site: int) -> float:
    """<psi| Z_site |psi> / <psi|psi> of an MPS in any gauge (Z = 2 S^z; `mpo` gives the physical
    legs): the network of the Z MPO by environment updates."""
    M = list(mps)
    if not M[0].data.is_complex():
        M = [BlockTensor(m.layout, m.data.to(torch.complex128)) for m in M]
    Lz, _ = _complex_envs(M, _aux_mpo("z", list(mpo), site))
    Ln, _ = _complex_envs(M, _aux_mpo("id", list(mpo)))
    return float(Lz[len(M)].data.sum().real / Ln[len(M)].data.sum().real)


def tdvp_observable_gradient(mps: Sequence[BlockTensor], mpo: Sequence[BlockTensor],
                             bond_op: Sequence[BlockTensor], chi: int, dt: float, n_steps: int,
                             site: int, **tdvp_kw):
    """<Z_site(t)> at t = n_steps dt after two-site TDVP from `mps`, and its derivatives with
    respect to the couplings J_i of H = sum_i J_i h_{i,i+1} (+ terms without J): `mpo` is H,
    `bond_op` the two-site MPO of h (e.g. `xxz_bond_operator`), Z = 2 S^z of a spin-1/2 S^z
    chain.

    Continuous adjoint: with psi(s) = exp(-iHs) psi(0) and lam(s) = exp(iH(t-s)) Z psi(t),
        d<Z(t)>/dJ_i = 2 int_0^t Im <lam(s)| h_i |psi(s)> ds.
    psi(s) comes from `tdvp2_evolve` with H, lam(s) from `tdvp2_evolve` of Z psi(t) with -H
    (states at every step kept on the device), the integrand from `im_transition_values`, the
    integral from `quadrature_weights`. Where the TDVP states are the exact ones (no truncation:
    chi above every bond's full dimension, Krylov exponentials converged) this is the exact
    derivative up to the quadrature error (Boole's rule: ~1e-10 relative at dt = 0.05, t = 1 on
    the XXZ chain); with truncation it is the derivative of the evolution the TDVP states
    approximate. Returns (value, gradient (N-1,), info)."""
    from .tdvp import tdvp2_evolve
    W = list(mpo)
    N = len(W)
    if not 0 <= site < N:
        raise ValueError(f"site {site} outside the chain")
    kw = dict(tdvp_kw)
    kw.pop("measure", None)
    kw.pop("meas_every", None)
    fwd, fwd_rec = tdvp2_evolve(list(mps), W, chi, dt, n_steps,
                                measure=clone_mps, meas_every=1, **kw)
    psi = [m for _, m in fwd_rec]
    W_neg = [BlockTensor(W[0].layout, -W[0].data)] + W[1:]
    lam_t = apply_pauli_z(psi[-1], site)
    _, bwd_rec = tdvp2_evolve(lam_t, W_neg, chi, dt, n_steps,
                              measure=clone_mps, meas_every=1, **kw)
    lam = [m for _, m in bwd_rec][::-1]
    W_id = _aux_mpo("id", W)
    value = z_expectation(psi[-1], W, site)
    g = np.stack([im_transition_values(lam[k], psi[k], W_id, bond_op)
                  for k in range(n_steps + 1)], axis=1)
    grad = 2.0 * g @ quadrature_weights(n_steps, dt)
    info = {"t": n_steps * dt, "points": n_steps + 1,
            "bond_dims": [int(m.legs[2].size) for m in psi[-1][:-1]]}
    return value, grad, info
