"""The per-sector Gram factorisation of the truncation (tnk_svd_gram_f64, the reference's
method='gram', tnkit/blocks.py:1345-1377) against numpy's SVD and the torch statement of the same
method: orthonormal factors, reconstruction, singular values in descending stable order, tall,
wide, square and one-row/one-column blocks."""
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


def _decaying(R, C, seed, span=6.0):
    rng = np.random.default_rng(seed)
    k = min(R, C)
    U, _ = np.linalg.qr(rng.standard_normal((R, k)))
    V, _ = np.linalg.qr(rng.standard_normal((C, k)))
    s = 10.0 ** (-np.linspace(0.0, span, k))
    return (U * s) @ V.T, s


@pytest.mark.parametrize("R,C", [(1, 1), (1, 7), (7, 1), (40, 40), (300, 120), (120, 300),
                                 (522, 519)])
def test_native_gram_matches_svd(R, C):
    from tnkit_gb300.linalg import _svd_gram, _svd_gram_native
    M, s = _decaying(R, C, R * 1000 + C)
    Md = torch.as_tensor(M, device="cuda")
    U, S, Vh, s_host = _svd_gram_native(Md)
    torch.cuda.synchronize()
    k = min(R, C)
    assert U.shape == (R, k) and S.shape == (k,) and Vh.shape == (k, C)
    Uh, Sh, Vhh = U.cpu().numpy(), S.cpu().numpy(), Vh.cpu().numpy()
    assert np.array_equal(Sh, s_host)
    assert np.all(np.diff(Sh) <= 0)
    # through the Gram matrix the values are exact to ~1e-16 of the largest squared
    assert np.abs(Sh - s).max() <= 1e-10 * s[0]
    assert np.abs(Uh.T @ Uh - np.eye(k)).max() <= 1e-12
    assert np.abs(Vhh @ Vhh.T - np.eye(k)).max() <= 1e-12
    # S = |diag R| drops R's off-diagonal; the reference's own bar for both methods is 1e-10 of
    # the largest value (tests/test_blocks.py:563-586)
    assert np.abs((Uh * Sh) @ Vhh - M).max() <= 1e-10 * s[0]
    # the torch statement of the same method gives the same factors up to column signs
    U2, S2, Vh2 = _svd_gram(Md)
    assert np.abs(S2.cpu().numpy() - Sh).max() <= 1e-10 * s[0]
    big = Sh > 1e-2 * Sh[0]          # vectors well separated at FP64 Gram precision
    for a, b in ((Uh[:, big], U2.cpu().numpy()[:, big]), (Vhh[big].T, Vh2.cpu().numpy()[big].T)):
        sg = np.sign(np.sum(a * b, axis=0))
        assert np.abs(a - b * sg).max() <= 1e-9


def test_native_gram_rejects_bad_workspace():
    import ctypes as C
    from tnkit_gb300 import _lib
    lib = _lib.lib()
    M = torch.ones((4, 3), dtype=torch.float64, device="cuda")
    out = torch.empty(64, dtype=torch.float64, device="cuda")
    ws = torch.empty(64, dtype=torch.uint8, device="cuda")
    nb = C.c_int64()
    assert lib.tnk_svd_gram_ws_f64(4, 3, C.byref(nb)) == 0 and nb.value > 64
    rc = lib.tnk_svd_gram_f64(M.data_ptr(), 4, 3, out.data_ptr(), out.data_ptr(),
                              out.data_ptr(), ws.data_ptr(), 64, None, _lib.stream_ptr())
    assert rc == _lib.TNK_ERR_SIZE


def test_truncated_svd_gram_native_matches_torch_path():
    """The bond truncation with the native factorisation keeps the same sectors and values as
    the torch statement of the method, and reconstructs the kept part."""
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(3)
    a = Leg((-1, 1), (5, 7), 1)
    b = Leg((-1, 1), (6, 4), -1)
    lay = layout_of((a, b), 0)
    h = rng.standard_normal(lay.size)
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    U, S, Vh, disc = LA.truncated_svd(m, 6, scale="none", method="gram")
    full = np.linalg.svd(h[:30].reshape(5, 6), compute_uv=False).tolist() + \
        np.linalg.svd(h[30:].reshape(7, 4), compute_uv=False).tolist()
    full = np.sort(full)[::-1]
    assert np.allclose(np.sort(S.cpu().numpy())[::-1], full[:6], rtol=1e-12, atol=0)
    assert abs(disc - float(np.sum(full[6:] ** 2))) <= 1e-12 * float(np.sum(full ** 2))


def test_host_split_matches_gpu_only():
    """The sectors split between the GPU and host LAPACK give the same truncation as all on the
    GPU or all on the host: kept values, bond sectors, discarded weight, reconstruction."""
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of, to_dense_np
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(9)
    a = Leg((-3, -1, 1, 3), (40, 260, 250, 30), 1)
    b = Leg((-3, -1, 1, 3), (35, 240, 255, 45), -1)
    lay = layout_of((a, b), 0)
    h = rng.standard_normal(lay.size) * np.repeat(
        10.0 ** -np.linspace(0, 4, lay.nblocks), [int(x) for x in lay.sizes])
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    res = {w: LA.truncated_svd(m, 300, scale="none", method="gram", host=w)
           for w in ("auto", "never", "always")}
    Ua, Sa, Va, da = res["never"]
    for w in ("auto", "always"):
        U, S, V, d = res[w]
        assert U.layout.legs == Ua.layout.legs and V.layout.legs == Va.layout.legs
        assert torch.allclose(S, Sa, rtol=1e-10, atol=1e-14 * float(Sa.max()))
        assert abs(d - da) <= 1e-10 * max(da, 1e-300) + 1e-24
        rec = to_dense_np(U.layout, U.data.cpu().numpy()) * S.cpu().numpy()[None, :] @ \
            to_dense_np(V.layout, V.data.cpu().numpy())
        rec0 = to_dense_np(Ua.layout, Ua.data.cpu().numpy()) * Sa.cpu().numpy()[None, :] @ \
            to_dense_np(Va.layout, Va.data.cpu().numpy())
        assert np.abs(rec - rec0).max() <= 1e-10 * float(Sa.max())


def test_fp32_truncation_close_to_fp64():
    """dtype=float32 (the opening sweeps of the mixed schedule): the same kept sectors, values
    within FP32-Gram accuracy, FP32-orthonormal factors returned in FP64."""
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of, to_dense_np
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(10)
    a = Leg((-1, 1), (150, 120), 1)
    b = Leg((-1, 1), (140, 130), -1)
    lay = layout_of((a, b), 0)
    h = rng.standard_normal(lay.size)
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    U, S, V, d = LA.truncated_svd(m, 60, scale="none", method="gram")
    U3, S3, V3, d3 = LA.truncated_svd(m, 60, scale="none", method="gram", dtype=torch.float32)
    assert U3.data.dtype == torch.float64 and U3.layout.legs == U.layout.legs
    assert float((S3 - S).abs().max()) <= 1e-5 * float(S.max())
    Ud = to_dense_np(U3.layout, U3.data.cpu().numpy())
    assert np.abs(Ud.T @ Ud - np.eye(Ud.shape[1])).max() <= 1e-5


@pytest.mark.parametrize("scale", ["right", "left"])
@pytest.mark.parametrize("host", ["never", "always"])
def test_direct_gram_side_matches_qr_form(scale, host):
    """The canonical side straight from its own Gram matrix (no QR) against the reference's
    QR form: the same kept values and bond, an orthonormal kept side, the same truncated
    matrix."""
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of, to_dense_np
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(12)
    a = Leg((-1, 1), (90, 120), 1)
    b = Leg((-1, 1), (100, 110), -1)
    lay = layout_of((a, b), 0)
    h = rng.standard_normal(lay.size) * np.repeat(10.0 ** -np.linspace(0, 3, lay.nblocks),
                                                   [int(x) for x in lay.sizes])
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    d = lambda t: to_dense_np(t.layout, t.data.cpu().numpy())
    U, S, V, disc = LA.truncated_svd(m, 80, scale=scale, method="gram", host=host)
    U0, S0, V0, disc0 = LA.truncated_svd(m, 80, scale=scale, method="gram", host=host,
                                         gram_qr=True)
    assert U.layout.legs == U0.layout.legs
    assert float((S - S0).abs().max()) <= 1e-10 * float(S0.max())
    assert abs(disc - disc0) <= 1e-9 * max(disc0, 1e-300)
    iso = d(U) if scale == "right" else d(V).T
    assert np.abs(iso.T @ iso - np.eye(iso.shape[1])).max() <= 1e-12
    assert np.abs(d(U) @ d(V) - d(U0) @ d(V0)).max() <= 1e-10
