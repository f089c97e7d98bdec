"""The host half of the device Gram truncation on the CPU: LAPACK's divide and conquer on
symmetric tridiagonals through scipy's Cython export (eigenvalues against numpy, orthonormal
vectors, graded DMRG-like spectra, orders 1 and 2, the threaded batch equal to one-by-one), and
the choice of a cluster size per sector order for the device reduction."""
import numpy as np
import pytest

pytest.importorskip("scipy")

from tnkit_gb300 import hostlapack


def _tri(n, seed, graded=False):
    rng = np.random.default_rng(seed)
    if graded:
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        G = (Q * 10.0 ** -np.linspace(0, 25, n)) @ Q.T
        from scipy.linalg import lapack
        _, d, e, _, info = lapack.dsytrd(G, lower=1)
        assert info == 0
        return d, e, np.linalg.eigvalsh(G)
    d, e = rng.standard_normal(n), rng.standard_normal(max(n - 1, 0))
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    return d, e, np.linalg.eigvalsh(T)


@pytest.mark.parametrize("n,graded", [(1, False), (2, False), (3, False), (40, False),
                                      (200, False), (300, True)])
def test_tridiag_eigh(n, graded):
    d, e, ref = _tri(n, n, graded)
    lam, Z = hostlapack.tridiag_eigh(d, e)
    assert lam.shape == (n,) and Z.shape == (n, n)
    assert np.all(np.diff(lam) >= 0)
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(lam - ref).max() <= 1e-13 * scale
    assert np.abs(Z.T @ Z - np.eye(n)).max() <= 1e-13
    T = np.diag(d) + np.diag(e[:n - 1], 1) + np.diag(e[:n - 1], -1)
    assert np.abs(T @ Z - Z * lam).max() <= 1e-13 * scale


def test_tridiag_eigh_many_equals_one_by_one():
    probs = [_tri(n, 7 + n)[:2] for n in (5, 120, 64, 1, 300, 33)]
    many = hostlapack.tridiag_eigh_many(probs, lanes=3)
    for (d, e), (lam, Z) in zip(probs, many):
        lam1, Z1 = hostlapack.tridiag_eigh(d, e)
        assert np.array_equal(lam, lam1) and np.array_equal(Z, Z1)


def test_cluster_choice():
    from tnkit_gb300 import linalg as LA
    saved = LA._SYTRD["limits"]
    LA._SYTRD["limits"] = {1: 168, 2: 238, 4: 335, 8: 470, 16: 660}
    try:
        mid = [522, 519, 344, 332, 142, 128, 31, 26, 2, 2]
        cs = LA._sytrd_clusters(mid, 152)
        assert all(LA._SYTRD["limits"][c] >= n for n, c in zip(mid, cs))
        assert cs[0] == 16 and cs[1] == 16 and sum(cs) <= 152
        many = LA._sytrd_clusters([100] * 400, 152)
        assert many == [1] * 400
        # a sector larger than every cluster size takes gets 0 (the caller's other route)
        assert LA._sytrd_clusters([700], 152) == [0]
    finally:
        LA._SYTRD["limits"] = saved


@pytest.mark.parametrize("n", [1, 2, 3, 50, 300])
def test_bidiag_svd(n):
    """dbdsdc through the Cython export: singular values against numpy (descending), orthonormal
    vectors, B = U diag(s) VT."""
    rng = np.random.default_rng(n)
    d = rng.standard_normal(n) * 10.0 ** -np.linspace(0, 8, n)
    e = rng.standard_normal(max(n - 1, 0)) * 10.0 ** -np.linspace(0, 8, max(n - 1, 0))
    B = np.diag(d) + (np.diag(e, 1) if n > 1 else 0)
    s, U, VT = hostlapack.bidiag_svd(d, e)
    ref = np.linalg.svd(B, compute_uv=False)
    assert np.all(np.diff(s) <= 0) and np.all(s >= 0)
    assert np.abs(s - ref).max() <= 1e-14 * max(ref[0], 1e-300)
    assert np.abs(U.T @ U - np.eye(n)).max() <= 1e-13
    assert np.abs(VT @ VT.T - np.eye(n)).max() <= 1e-13
    assert np.abs((U * s) @ VT - B).max() <= 1e-14 * max(ref[0], 1e-300)


def test_bidiag_svd_many_equals_one_by_one():
    rng = np.random.default_rng(3)
    probs = [(rng.standard_normal(n), rng.standard_normal(max(n - 1, 0))) for n in (7, 90, 1, 33)]
    many = hostlapack.bidiag_svd_many(probs, lanes=3)
    for (d, e), (s, U, VT) in zip(probs, many):
        s1, U1, VT1 = hostlapack.bidiag_svd(d, e)
        assert np.array_equal(s, s1) and np.array_equal(U, U1) and np.array_equal(VT, VT1)


def test_exact_route_cluster_choice():
    from tnkit_gb300 import linalg as LA
    saved = LA._GEBRD["limits"]
    LA._GEBRD["limits"] = {1: 160, 2: 228, 4: 322, 8: 450, 16: 630}
    try:
        shapes = [(522, 519), (344, 344), (142, 142), (31, 31), (2, 2)]
        cs = LA._gebrd_clusters(shapes, 152)
        assert all(LA._GEBRD["limits"][c] >= m for (m, _), c in zip(shapes, cs))
        assert cs[0] == 16 and sum(cs) <= 152
        assert LA._gebrd_clusters([(700, 10)], 152) == [0]
    finally:
        LA._GEBRD["limits"] = saved
