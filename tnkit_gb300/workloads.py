"""Synthetic chains and local problems with the shapes of the benchmark configurations.

  xxz_mpo(N, delta)     open spin-1/2 XXZ chain, H = sum (S+S- + S-S+)/2 + delta SzSz, MPO width 5
                        (the bulk tensor of the reference's bench/profile/fused_dmrg_check.py:48-53)
  tfim_mpo(N, g)        open transverse-field Ising chain, H = -sum XX - g sum Z, width 3
                        (tnkit/models.py:50-95 with h = 0)
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


def tfim_mpo(N: int, g: float = 1.0):
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sz = np.diag([1.0, -1.0])
    W = np.zeros((3, 3, 2, 2))
    W[0, 0], W[0, 1], W[0, 2], W[1, 2], W[2, 2] = np.eye(2), sx, -g * sz, -sx, np.eye(2)
    return open_chain(W, N)


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
