"""tnkit_gb300: the DMRG/TDVP inner loop of tnkit, GB300-native (sm_103a).

The two-site effective-Hamiltonian matvec, the one-site matvec and the left/right environment
updates run as hand-written CUDA kernels over the reference's canonical block-sparse layout,
called through a C ABI (include/tnkit_gb300.h). The Krylov solvers and the sweep around them
keep their vectors on the GPU and call the same library for their reductions.

Public surface (mirrors the reference's names):
  apply_two_site, apply_one_site, update_left_env, update_right_env   (tnkit/_dmrg.py:162-231)
  lanczos_ground_restart                                              (tnkit/eigensolver.py:507)
  dmrg, DMRGOptions                                                   (tnkit/_dmrg.py:312-522)
  to_block_mpo, random_block_mps                                      (tnkit/block_backend.py)
  get_backend("b200"), B200Backend
"""
from .layout import Leg, Layout, canonical, layout_of
from .tensor import BlockTensor
from ._lib import LibraryMissing, TnkError

__version__ = "0.1.0"


def __getattr__(name):
    # Heavy modules (torch) load on first use, so `import tnkit_gb300` stays cheap.
    if name in ("apply_two_site", "apply_one_site", "update_left_env", "update_right_env",
                "tensordot", "TwoSiteOperator"):
        from . import ops
        return getattr(ops, name)
    if name in ("to_block_mpo", "random_block_mps", "mpo_charges", "dense_mpo",
                "random_dense_mps"):
        from . import mpo
        return getattr(mpo, name)
    if name in ("lanczos_ground_restart",):
        from . import lanczos
        return getattr(lanczos, name)
    if name in ("dmrg", "DMRGOptions"):
        from . import dmrg as _d
        return getattr(_d, name)
    if name in ("get_backend", "B200Backend"):
        from . import backend
        return getattr(backend, name)
    raise AttributeError(name)
