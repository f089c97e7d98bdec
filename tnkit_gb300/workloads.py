"""Synthetic chains and local problems with the shapes of the benchmark configurations.

  xxz_mpo(N, delta)     open spin-1/2 XXZ chain, H = sum (S+S- + S-S+)/2 + delta SzSz, MPO width 5
                        (the bulk tensor of the reference's bench/profile/fused_dmrg_check.py:48-53)
  tfim_mpo(N, g)        open transverse-field Ising chain, H = -sum XX - g sum Z, width 3
                        (tnkit/models.py:50-95 with h = 0)
  hubbard_mpo(N, t, U)  open Fermi-Hubbard chain H = -t sum (c+_{i s} c_{i+1 s} + h.c.)
                        + U sum n_{i up} n_{i dn}, one d=4 site per orbital (|0>, |up>, |dn>,
                        |up dn>), Jordan-Wigner strings inside the MPO, width 6; site charges
                        (N_up, N_dn) for U(1) x U(1) blocks (HUBBARD_SITE_CHARGES)
  mid_bond_problem      random U(1) environments and two-site block of a chain's bond, with given
                        sector dims: the local problem one Lanczos matvec sees.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from .layout import Leg, layout_of
from .mpo import to_block_mpo
from .tensor import BlockTensor

# Sector dims of the mid bond of the U(1) XXZ N=64 chain at chi=1024 (converged reference run):
# 2 S^z = -8 .. 8 step 2.
C2_MID_CHARGES = (-8, -6, -4, -2, 0, 2, 4, 6, 8)
C2_MID_DIMS = (2, 29, 113, 231, 291, 228, 104, 24, 2)


def xxz_bulk(delta: float = 1.0) -> np.ndarray:
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm, sz, i2 = sp.T.copy(), np.diag([0.5, -0.5]), np.eye(2)
    W = np.zeros((5, 5, 2, 2))
    W[0, 0], W[0, 1], W[0, 2], W[0, 3] = i2, sp, sm, sz
    W[1, 4], W[2, 4], W[3, 4], W[4, 4] = 0.5 * sm, 0.5 * sp, delta * sz, i2
    return W


def open_chain(Wb: np.ndarray, N: int):
    D = Wb.shape[0]
    return [Wb[0:1] if i == 0 else Wb[:, D - 1:D] if i == N - 1 else Wb for i in range(N)]


def xxz_mpo(N: int, delta: float = 1.0):
    return open_chain(xxz_bulk(delta), N)


def xxz_disordered_mpo(J: Sequence[float], delta: float = 1.0):
    """Open XXZ chain H = sum_i J_i [(S+S- + S-S+)/2 + delta Sz Sz]_{i,i+1} with one coupling per
    bond (len(J) = N - 1): the bond's J_i sits on the left site's outgoing channels."""
    N = len(J) + 1
    out = []
    for i in range(N):
        W = xxz_bulk(delta)
        j = J[i] if i < N - 1 else 1.0
        W[0, 1:4] *= j
        out.append(W[0:1] if i == 0 else W[:, 4:5] if i == N - 1 else W)
    return out


def tfim_mpo(N: int, g: float = 1.0):
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sz = np.diag([1.0, -1.0])
    W = np.zeros((3, 3, 2, 2))
    W[0, 0], W[0, 1], W[0, 2], W[1, 2], W[2, 2] = np.eye(2), sx, -g * sz, -sx, np.eye(2)
    return open_chain(W, N)


# (N_up, N_dn) of the local states |0>, |up>, |dn>, |up dn>
HUBBARD_SITE_CHARGES = ((0, 0), (1, 0), (0, 1), (1, 1))


def hubbard_bulk(t: float = 1.0, U: float = 4.0) -> np.ndarray:
    """Bulk MPO tensor (6, 6, 4, 4) of the Fermi-Hubbard chain. The fermions are ordered
    (1 up, 1 dn, 2 up, 2 dn, ...) with Jordan-Wigner strings: with hard-core a_s on a site,
    F_s = (-1)^n_s and F = F_up F_dn, c+_{j up} c_{j+1 up} = (a+_up F)_j (a_up)_{j+1},
    c+_{j+1 up} c_{j up} = (F a_up)_j (a+_up)_{j+1}, c+_{j dn} c_{j+1 dn} =
    (F_up a+_dn F)_j (F_up a_dn)_{j+1}, c+_{j+1 dn} c_{j dn} = (F F_up a_dn)_j (F_up a+_dn)_{j+1}.
    Channels: idle, the four hops, done."""
    e = lambda i, j: np.outer(np.eye(4)[i], np.eye(4)[j])
    a_up = e(0, 1) + e(2, 3)
    a_dn = e(0, 2) + e(1, 3)
    n_up, n_dn = np.diag([0.0, 1.0, 0.0, 1.0]), np.diag([0.0, 0.0, 1.0, 1.0])
    f_up, f_dn = np.diag([1.0, -1.0, 1.0, -1.0]), np.diag([1.0, 1.0, -1.0, -1.0])
    f = f_up @ f_dn
    i4 = np.eye(4)
    W = np.zeros((6, 6, 4, 4))
    W[0, 0], W[5, 5] = i4, i4
    W[0, 1], W[1, 5] = a_up.T @ f, -t * a_up
    W[0, 2], W[2, 5] = f @ a_up, -t * a_up.T
    W[0, 3], W[3, 5] = f_up @ a_dn.T @ f, -t * f_up @ a_dn
    W[0, 4], W[4, 5] = f @ f_up @ a_dn, -t * f_up @ a_dn.T
    W[0, 5] = U * n_up @ n_dn
    return W


def hubbard_mpo(N: int, t: float = 1.0, U: float = 4.0):
    return open_chain(hubbard_bulk(t, U), N)


def mid_bond_problem(charges: Sequence[int] = C2_MID_CHARGES,
                     dims: Sequence[int] = C2_MID_DIMS, seed: int = 0, device="cuda",
                     N: int = 8, delta: float = 1.0):
    """(theta, L, W1, W2, R) of a bulk bond of the U(1) XXZ chain whose left and right bonds have
    the given sectors (the same on both sides), random entries from `seed`."""
    Wb, _ = to_block_mpo(xxz_mpo(N, delta), [[1, -1]] * N, device=device)
    W1, W2 = Wb[N // 2 - 1], Wb[N // 2]
    bond = Leg(tuple(int(c) for c in charges), tuple(int(d) for d in dims), 1)
    phys = W1.legs[2]
    rng = np.random.default_rng(seed)
    th_l = layout_of((bond, phys, phys, bond.flip()), 0)
    L_l = layout_of((bond, W1.legs[0].flip(), bond.flip()), 0)
    R_l = layout_of((bond.flip(), W2.legs[1].flip(), bond), 0)

    def rnd(lay):
        h = rng.standard_normal(lay.size)
        return BlockTensor(lay, torch.as_tensor(h, device=device), h)
    return rnd(th_l), rnd(L_l), W1, W2, rnd(R_l)
