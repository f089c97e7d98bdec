"""The device tridiagonal eigensolver (tnk_tridiag_eig_f64, implicit QL) against numpy's
dense symmetric eigensolver, and the backend's Krylov exponential step built on it
(expm_sym_tridiag_eigh, tnkit/backend.py:643-661) against scipy's expm."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


def _cases(seed):
    rng = np.random.default_rng(seed)
    out = []
    for n in (1, 2, 3, 7, 17, 31, 32, 40, 41, 64, 100, 128):
        d = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3)
        e = rng.standard_normal(n - 1) * 10.0 ** rng.uniform(-8, 2)
        out.append((d, e))
    # split blocks, a constant diagonal (clustered spectrum), a graded Lanczos-like matrix
    d = np.ones(30)
    e = rng.standard_normal(29) * 1e-3
    e[[5, 11, 12, 20]] = 0.0
    out.append((d, e))
    out.append((np.full(16, 2.5), np.zeros(15)))
    j = np.arange(40)
    out.append((-2.0 + 0.01 * j, 10.0 ** (-j[:-1] / 6.0)))
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_tridiag_eigh_matches_dense_eigensolver(seed):
    from tnkit_gb300.tridiag import tridiag_eigh_batched
    for d, e in _cases(seed):
        n = len(d)
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        lam, V = tridiag_eigh_batched(torch.as_tensor(d[None], device="cuda"),
                                      torch.as_tensor(e[None], device="cuda") if n > 1 else None)
        lam, V = lam[0].cpu().numpy(), V[0].cpu().numpy()
        ref = np.linalg.eigvalsh(T)
        sc = max(np.abs(ref).max(), 1e-300)
        assert np.all(np.diff(lam) >= 0)
        assert np.abs(lam - ref).max() <= 1e-13 * sc, (n, np.abs(lam - ref).max() / sc)
        assert np.abs(T @ V - V * lam).max() <= 1e-13 * sc
        assert np.abs(V.T @ V - np.eye(n)).max() <= 1e-13


def test_tridiag_batched_launch_equals_one_by_one():
    from tnkit_gb300.tridiag import tridiag_eigh_batched
    rng = np.random.default_rng(5)
    k, m = 9, 24
    d = torch.as_tensor(rng.standard_normal((k, m)), device="cuda")
    e = torch.as_tensor(rng.standard_normal((k, m - 1)), device="cuda")
    lam, V = tridiag_eigh_batched(d, e)
    for b in range(k):
        l1, v1 = tridiag_eigh_batched(d[b:b + 1], e[b:b + 1])
        assert torch.equal(l1[0], lam[b]) and torch.equal(v1[0], V[b])


def test_expm_sym_tridiag_eigh_matches_scipy():
    from scipy.linalg import expm
    from tnkit_gb300.backend import get_backend
    be = get_backend("b200")
    rng = np.random.default_rng(3)
    for m in (1, 5, 17, 30):
        d = rng.standard_normal(m)
        e = np.abs(rng.standard_normal(m - 1))
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        tau = -0.5j * 0.05
        got = be.expm_sym_tridiag_eigh(torch.as_tensor(d, device="cuda"),
                                       torch.as_tensor(e, device="cuda") if m > 1 else None, tau)
        assert np.abs(got.cpu().numpy() - expm(tau * T)).max() <= 1e-13
    dd = torch.as_tensor(rng.standard_normal((4, 12)), device="cuda")
    ee = torch.as_tensor(np.abs(rng.standard_normal((4, 11))), device="cuda")
    out = be.expm_sym_tridiag_eigh_batched(dd, ee, 0.3j)
    for b in range(4):
        T = np.diag(dd[b].cpu().numpy()) + np.diag(ee[b].cpu().numpy(), 1) + \
            np.diag(ee[b].cpu().numpy(), -1)
        assert np.abs(out[b].cpu().numpy() - expm(0.3j * T)).max() <= 1e-13


def test_tridiag_rejects_bad_orders():
    from tnkit_gb300 import _lib
    from tnkit_gb300.tridiag import tridiag_eigh_batched
    with pytest.raises(ValueError):
        tridiag_eigh_batched(torch.zeros((1, 129), dtype=torch.float64, device="cuda"),
                             torch.zeros((1, 128), dtype=torch.float64, device="cuda"))
    lib = _lib.lib()
    assert lib.tnk_tridiag_eig_f64(None, None, 0, 1, 1, 1, None, None, None, None) == \
        _lib.TNK_ERR_ARG
