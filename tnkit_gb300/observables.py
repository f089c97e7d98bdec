"""Schmidt spectra and entanglement entropies of a block MPS on the GPU.

  schmidt_spectra   tnkit/observables.py:313-338 (_schmidt_sweep): right-canonicalise a copy,
                    carry the orthogonality centre left to right, and read every bond's singular
                    values off the SVD that moves it
  all_entropies     tnkit/observables.py:373-387 with _entropy (:341-347): the spectrum
                    normalised, p = s^2, only p > 1e-16 counted, S = -sum p ln p (natural log)

The reference computes a block state's entropies on its dense form (to_dense_mps, then the dense
sweep); here the sweep runs on the blocks themselves: the singular values of a block matrix are
those of its dense form (the blocks are its charge sectors), so the spectra agree up to their
order, which the entropy does not see. Every SVD is the exact per-sector route
(`linalg.truncated_svd` with method='svd' and nothing cut); the contractions are the library's
block tensordot. The state is not modified.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np
import torch

from . import linalg as LA
from . import ops
from .tensor import BlockTensor


def _entropy(s: np.ndarray) -> float:
    """Von Neumann entropy of one Schmidt spectrum, normalised here (tnkit/observables.py:341)."""
    s = np.asarray(s, dtype=np.float64)
    nrm = np.linalg.norm(s)
    if nrm == 0.0:
        raise ValueError("a bond with an all-zero Schmidt spectrum")
    p = (s / nrm) ** 2
    p = p[p > 1e-16]
    return float(-np.sum(p * np.log(p)))


def schmidt_spectra(mps: Sequence[BlockTensor]) -> List[np.ndarray]:
    """Every bond's Schmidt values (host arrays, descending), bond i between sites i and i+1."""
    from .dmrg import right_canonicalize
    if len(mps) < 2:
        return []
    dev = mps[0].data.device
    M = right_canonicalize([BlockTensor(m.layout, m.data.clone()) for m in mps],
                           LA.Scalars(dev))
    out = []
    carry = None
    for i in range(len(M) - 1):
        A = M[i] if carry is None else ops.tensordot(carry, M[i], 1)
        mat, info = LA.fuse_matrix(A, 2)
        big = sum(int(l.size) for l in mat.legs)
        U, S, Vh, _ = LA.truncated_svd(mat, big, scale="right", method="svd", normalize=False)
        out.append(np.sort(S.detach().cpu().numpy().astype(np.float64))[::-1].copy())
        carry = LA.split_cols(Vh, info)     # S Vh: the centre on the bond, legs (bond, b)
    return out


def all_entropies(mps: Sequence[BlockTensor]) -> np.ndarray:
    """Every bond's entanglement entropy (array of N - 1), as the reference's all_entropies."""
    return np.array([_entropy(s) for s in schmidt_spectra(mps)])
