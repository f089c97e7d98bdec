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
