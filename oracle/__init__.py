"""CPU oracle for the DMRG/TDVP inner loop -- TEST INFRASTRUCTURE, not part of the product.

A plain numpy restatement of the reference algorithms on the hot path (tnkit 0.3.0):
block-sparse abelian tensors in the reference's canonical layout, the two-site and one-site
effective-Hamiltonian matvecs, the left/right environment updates, thick-restart Lanczos, the
block truncated SVD and the two-site DMRG sweep. Each function cites the reference file:line it
restates.

Only `tests/`, `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` may import this
package, and only as the checker (or the timed CPU baseline), never as the thing measured or
shipped. The product package `tnkit_gb300` never imports it.

Parity is pinned: `tests/test_oracle_golden.py` checks every function here against golden
vectors produced by running the reference itself (`tests/golden/make_golden.py`).
"""
