"""The device Gram route of the truncation (tnk_sytrd_batched_f64 / tnk_ormtr_batched_f64 with
the host tridiagonal solver between them) against numpy and against the cuSOLVER route:
tridiagonal reductions with the Gram matrix's eigenvalues, orthonormal back-transformed
eigenvectors that reconstruct it, the same kept values, bond sectors and discarded weight as
the per-sector cuSOLVER factorisation, and DMRG on it matching the reference's energies."""
import ctypes as C
import importlib
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()
    from tnkit_gb300 import linalg as LA
    if not LA.device_gram_available():
        pytest.fail("the device Gram route is unavailable on this device")


def _gram(n, seed, span=30.0):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = 10.0 ** (-np.linspace(0.0, span, n))
    return (Q * lam) @ Q.T, lam


@pytest.mark.parametrize("cs", [1, 2, 4, 8, 16])
def test_reduction_and_back_transformation(cs):
    """Several sectors of different orders in one launch each, on clusters of cs CTAs: T's
    eigenvalues are G's to FP64 accuracy, Q Z is orthonormal and reconstructs G."""
    from tnkit_gb300 import _lib, hostlapack
    from tnkit_gb300 import linalg as LA
    lib = _lib.lib()
    nmax = LA._sytrd_table()[cs]
    if nmax == 0:
        pytest.skip(f"clusters of {cs} cannot launch here")
    orders = [n for n in (1, 2, 3, 17, 100, 33, 522, 640) if n <= nmax] + [nmax]
    gs = [_gram(n, 100 + n) for n in orders]
    tab = np.zeros((len(orders), 4), np.int64)
    g = v = 0
    for r, n in enumerate(orders):
        tab[r, :3] = (n, g, v)
        g += n * n
        v += n
    G = torch.as_tensor(np.concatenate([x[0].T.reshape(-1) for x in gs]), device="cuda")
    dv = torch.zeros(3 * v, dtype=torch.float64, device="cuda")
    tab_d = torch.as_tensor(tab, device="cuda")
    sp = _lib.stream_ptr()
    _lib.check(lib.tnk_sytrd_batched_f64(tab_d.data_ptr(), len(orders), max(orders), cs,
                                         G.data_ptr(), dv.data_ptr(), dv.data_ptr() + 8 * v,
                                         dv.data_ptr() + 16 * v, sp), "sytrd")
    dh = dv.cpu().numpy()
    zs, items = [], []
    z = 0
    lams = []
    for r, n in enumerate(orders):
        d, e = dh[tab[r, 2]:tab[r, 2] + n], dh[v + tab[r, 2]:v + tab[r, 2] + n]
        lam, Z = hostlapack.tridiag_eigh(d, e)
        lams.append(lam)
        ref = np.linalg.eigvalsh(gs[r][0])
        assert np.abs(lam - ref).max() <= 1e-14, n
        tab[r, 3] = z
        zs.append(np.asfortranarray(Z).T.reshape(-1))        # column-major n x n
        for c0 in range(0, n, 8):
            items.append((r, c0, min(8, n - c0), 0))
        z += n * n
    Zd = torch.as_tensor(np.concatenate(zs), device="cuda")
    tab_d = torch.as_tensor(tab, device="cuda")
    it_d = torch.as_tensor(np.asarray(items, np.int32), device="cuda")
    _lib.check(lib.tnk_ormtr_batched_f64(tab_d.data_ptr(), it_d.data_ptr(), len(items),
                                         max(orders), G.data_ptr(), dv.data_ptr() + 16 * v,
                                         Zd.data_ptr(), sp), "ormtr")
    Zh = Zd.cpu().numpy()
    for r, n in enumerate(orders):
        U = Zh[tab[r, 3]:tab[r, 3] + n * n].reshape(n, n).T      # columns: eigenvectors of G
        assert np.abs(U.T @ U - np.eye(n)).max() <= 1e-13, n
        assert np.abs((U * lams[r]) @ U.T - gs[r][0]).max() <= 1e-14, n


def test_sytrd_rejects_oversize_order():
    from tnkit_gb300 import _lib
    from tnkit_gb300 import linalg as LA
    lib = _lib.lib()
    cs, nmax = LA._sytrd_limits()
    rc = lib.tnk_sytrd_batched_f64(8, 1, nmax + 64, cs, 8, 8, 8, 8, None)
    assert rc == _lib.TNK_ERR_SIZE


def _mid_bond_matrix(seed):
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300 import workloads
    from tnkit_gb300.tensor import BlockTensor
    th, *_ = workloads.mid_bond_problem(seed=seed, device="cuda")
    rng = np.random.default_rng(seed)
    x = torch.as_tensor(rng.standard_normal(th.layout.size), device="cuda")
    mat, info = LA.fuse_matrix(BlockTensor(th.layout, x / x.norm()), 2)
    return mat


@pytest.mark.parametrize("scale", ["right", "left", "none"])
def test_device_route_matches_cusolver_route(scale):
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of, to_dense_np
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(21)
    a = Leg((-2, 0, 2), (60, 310, 140), 1)
    b = Leg((-2, 0, 2), (70, 300, 150), -1)
    lay = layout_of((a, b), 0)
    h = rng.standard_normal(lay.size) * np.repeat(10.0 ** -np.linspace(0, 3, lay.nblocks),
                                                   [int(x) for x in lay.sizes])
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    dn = lambda t: to_dense_np(t.layout, t.data.cpu().numpy())
    U, S, V, disc = LA.truncated_svd(m, 250, scale=scale, method="gram", host="device")
    U0, S0, V0, disc0 = LA.truncated_svd(m, 250, scale=scale, method="gram", host="never")
    assert U.layout.legs == U0.layout.legs and V.layout.legs == V0.layout.legs
    assert float((S - S0).abs().max()) <= 1e-10 * float(S0.max())
    assert abs(disc - disc0) <= 1e-9 * max(disc0, 1e-300)
    if scale == "right":
        iso = dn(U)
    elif scale == "left":
        iso = dn(V).T
    else:
        iso = dn(U) if dn(U).shape[0] <= dn(V).shape[1] else dn(V).T
    assert np.abs(iso.T @ iso - np.eye(iso.shape[1])).max() <= 1e-12
    mid = np.ones_like(S.cpu().numpy()) if scale != "none" else S.cpu().numpy()
    assert np.abs((dn(U) * mid) @ dn(V) - (dn(U0) * mid) @ dn(V0)).max() <= 1e-10


def test_device_route_many_matches_one_by_one():
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(5)
    mats = []
    for k in range(3):
        a = Leg((-1, 1), (30 + 10 * k, 50), 1)
        b = Leg((-1, 1), (40, 45 + 5 * k), -1)
        lay = layout_of((a, b), 0)
        h = rng.standard_normal(lay.size)
        mats.append(BlockTensor(lay, torch.as_tensor(h, device="cuda"), h))
    many = LA.truncated_svd_many([(m, 40, "right") for m in mats], method="gram", host="device")
    for m, (U, S, V, d) in zip(mats, many):
        U1, S1, V1, d1 = LA.truncated_svd(m, 40, scale="right", method="gram", host="device")
        assert U.layout.legs == U1.layout.legs
        assert torch.allclose(S, S1, rtol=1e-13, atol=0)
        assert torch.allclose(U.data, U1.data, rtol=0, atol=1e-12)
        assert torch.allclose(V.data, V1.data, rtol=0, atol=1e-12)
        assert abs(d - d1) <= 1e-13 * max(d1, 1e-300)


def test_mid_bond_truncation_device_route():
    """The chi=1024 mid-bond block (XXZ N=64 sectors, up to 522 rows): the device route keeps the
    same values and sectors as the cuSOLVER route."""
    from tnkit_gb300 import linalg as LA
    mat = _mid_bond_matrix(3)
    U, S, V, disc = LA.truncated_svd(mat, 1024, scale="right", method="gram", host="device")
    U0, S0, V0, disc0 = LA.truncated_svd(mat, 1024, scale="right", method="gram", host="never")
    assert U.layout.legs == U0.layout.legs
    assert float((S**2 - S0**2).abs().max()) <= 1e-13 * float(S0.max() ** 2)
    assert abs(disc - disc0) <= 1e-12


@pytest.mark.parametrize("N,chi", [(12, 64), (64, 64)])
def test_dmrg_on_device_route_matches_reference(N, chi):
    """DMRG with the Gram truncation on the device route: the reference's exact-SVD energy to
    1e-10 (the bar of the cuSOLVER Gram route) and every bond's sectors."""
    D = importlib.import_module("tnkit_gb300.dmrg")
    from tnkit_gb300 import workloads
    from tnkit_gb300.mpo import to_block_mpo
    ref = json.load(open(os.path.join(GOLDEN, "dmrg_small.json")))[f"xxz_n{N}_chi{chi}"]
    Wb = to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N)[0]
    E, M, info = D.dmrg(Wb, chi, charge=0, seed=1, n_sweeps=len(ref["energies"]), tol=0,
                        rtol=0, expand=0, svd_method="gram", svd_host="device")
    assert abs(E - ref["E"]) <= 1e-10, (E, ref["E"])
    for m, b in zip(M, ref["bonds"]):
        assert list(m.legs[2].dims) == b["dims"] and list(m.legs[2].charges) == b["charges"]


# ---- the exact route (method='svd') ---------------------------------------------------------

def _graded(R, C, seed, span=12.0):
    rng = np.random.default_rng(seed)
    k = min(R, C)
    U, _ = np.linalg.qr(rng.standard_normal((R, k)))
    V, _ = np.linalg.qr(rng.standard_normal((C, k)))
    s = 10.0 ** (-np.linspace(0.0, span, k))
    return (U * s) @ V.T, s


@pytest.mark.parametrize("cs", [1, 4, 16])
def test_bidiagonalisation_and_back_transformation(cs):
    """Blocks of several shapes (tall, wide through the transpose, square, one row/column) in one
    launch: B's singular values are the block's to FP64 accuracy, the back-transformed vectors
    are orthonormal and reconstruct the block."""
    from tnkit_gb300 import _lib, hostlapack
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300._lib import GEBRD_SECTOR, REFL_SET
    lib = _lib.lib()
    mmax = LA._gebrd_table()[cs]
    if mmax == 0:
        pytest.skip(f"clusters of {cs} cannot launch here")
    shapes = [(s0, s1) for s0, s1 in ((1, 1), (5, 1), (1, 4), (3, 3), (40, 17), (17, 40),
                                      (130, 100), (300, 300), (mmax, mmax - 7))
              if max(s0, s1) <= mmax]
    mats = [_graded(R, C, 7 + R + 3 * C)[0] for R, C in shapes]
    buf = np.concatenate([M.reshape(-1) for M in mats])
    Md = torch.as_tensor(buf, device="cuda")
    tab = np.zeros(len(shapes), dtype=GEBRD_SECTOR)
    a = refl = vo = 0
    for r, (R, C) in enumerate(shapes):
        tr = R < C
        mm, nn = max(R, C), min(R, C)
        tab[r] = (mm, nn, a, refl, refl + mm * nn, vo, 0, 1 if tr else C, C if tr else 1)
        a += R * C
        refl += mm * nn + nn * nn
        vo += 4 * nn
    RF = torch.zeros(refl, dtype=torch.float64, device="cuda")
    vec = torch.zeros(vo, dtype=torch.float64, device="cuda")
    tab_d = torch.as_tensor(tab.view(np.uint8), device="cuda")
    sp = _lib.stream_ptr()
    _lib.check(lib.tnk_gebrd_batched_f64(tab_d.data_ptr(), len(shapes), int(tab["m"].max()),
                                         int(tab["n"].max()), cs, Md.data_ptr(), RF.data_ptr(),
                                         RF.data_ptr(), vec.data_ptr(), sp), "gebrd")
    vh = vec.cpu().numpy()
    sets, items, zs, z = [], [], [], 0
    res = []
    for r, (R, C) in enumerate(shapes):
        mm, nn, v0 = int(tab[r]["m"]), int(tab[r]["n"]), int(tab[r]["v_off"])
        s, Ub, VTb = hostlapack.bidiag_svd(vh[v0:v0 + nn], vh[v0 + nn:v0 + 2 * nn])
        ref = np.linalg.svd(mats[r], compute_uv=False)
        assert np.abs(s - ref).max() <= 1e-13 * ref[0], (R, C)
        res.append(s)
        zl = np.zeros((nn, mm))
        zl[:, :nn] = Ub.T
        zs += [zl.reshape(-1), np.ascontiguousarray(VTb).reshape(-1)]
        sets.append((mm, nn, int(tab[r]["ul_off"]), v0 + 2 * nn, z, 0, 0))
        sets.append((nn, max(nn - 2, 0), int(tab[r]["vr_off"]), v0 + 3 * nn, z + mm * nn, 1, 0))
        for si in (len(sets) - 2, len(sets) - 1):
            for c0 in range(0, nn, 8):
                items.append((si, c0, min(8, nn - c0), 0))
        z += (mm + nn) * nn
    st = np.zeros(len(sets), dtype=REFL_SET)
    arr = np.asarray(sets, dtype=np.int64)
    for f, name in enumerate(("rows", "nrefl", "r_off", "tau_off", "z_off", "shift", "pad")):
        st[name] = arr[:, f]
    Zd = torch.as_tensor(np.concatenate(zs), device="cuda")
    st_d = torch.as_tensor(st.view(np.uint8), device="cuda")
    it_d = torch.as_tensor(np.asarray(items, np.int32), device="cuda")
    _lib.check(lib.tnk_ormqr_batched_f64(st_d.data_ptr(), it_d.data_ptr(), len(items),
                                         int(st["rows"].max()), RF.data_ptr(), vec.data_ptr(),
                                         Zd.data_ptr(), sp), "ormqr")
    Zh = Zd.cpu().numpy()
    for r, (R, C) in enumerate(shapes):
        mm, nn = int(tab[r]["m"]), int(tab[r]["n"])
        zl, zr = int(st[2 * r]["z_off"]), int(st[2 * r + 1]["z_off"])
        Lq = Zh[zl:zl + mm * nn].reshape(nn, mm).T
        Rq = Zh[zr:zr + nn * nn].reshape(nn, nn).T
        U, V = (Lq, Rq) if R >= C else (Rq, Lq)
        assert np.abs(U.T @ U - np.eye(nn)).max() <= 1e-13, (R, C)
        assert np.abs(V.T @ V - np.eye(nn)).max() <= 1e-13, (R, C)
        assert np.abs((U * res[r]) @ V.T - mats[r]).max() <= 1e-13, (R, C)


@pytest.mark.parametrize("scale", ["right", "left", "none"])
def test_exact_device_route_matches_torch_svd(scale):
    """truncated_svd(method='svd') on the device route against torch.linalg.svd per sector:
    the same kept values (1e-13 of the largest), bond, discarded weight (1e-12 of the total) and
    truncated matrix; orthonormal factors."""
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of, to_dense_np
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(31)
    a = Leg((-2, 0, 2), (60, 310, 140), 1)
    b = Leg((-2, 0, 2), (70, 300, 150), -1)
    lay = layout_of((a, b), 0)
    h = rng.standard_normal(lay.size) * np.repeat(10.0 ** -np.linspace(0, 3, lay.nblocks),
                                                   [int(x) for x in lay.sizes])
    h /= np.linalg.norm(h)
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    dn = lambda t: to_dense_np(t.layout, t.data.cpu().numpy())
    U, S, V, disc = LA.truncated_svd(m, 250, scale=scale, method="svd", host="device")
    U0, S0, V0, disc0 = LA.truncated_svd(m, 250, scale=scale, method="svd", host="never")
    assert U.layout.legs == U0.layout.legs and V.layout.legs == V0.layout.legs
    assert float((S - S0).abs().max()) <= 1e-13 * float(S0.max())
    assert abs(disc - disc0) <= 1e-12
    mid = np.ones_like(S.cpu().numpy()) if scale != "none" else S.cpu().numpy()
    assert np.abs((dn(U) * mid) @ dn(V) - (dn(U0) * mid) @ dn(V0)).max() <= 1e-12
    iso = dn(U) if scale != "left" else dn(V).T
    assert np.abs(iso.T @ iso - np.eye(iso.shape[1])).max() <= 1e-12


def test_exact_device_route_mid_bond():
    """The chi=1024 mid-bond block on the exact device route: the same spectrum as
    torch.linalg.svd per sector to 1e-14 of the largest value."""
    from tnkit_gb300 import linalg as LA
    mat = _mid_bond_matrix(5)
    U, S, V, disc = LA.truncated_svd(mat, 1024, scale="right", method="svd", host="device")
    U0, S0, V0, disc0 = LA.truncated_svd(mat, 1024, scale="right", method="svd", host="never")
    assert U.layout.legs == U0.layout.legs
    assert float((S - S0).abs().max()) <= 1e-14 * float(S0.max()) * 10
    assert abs(disc - disc0) <= 1e-12


@pytest.mark.parametrize("method", ["gram", "svd"])
def test_sectors_above_the_cluster_limit_take_the_library_route(method, monkeypatch):
    """With the cluster kernels' order limit lowered below the largest sector, that sector goes
    through the per-sector library route (cuSOLVER Gram / torch SVD) and the rest through the
    device kernels, in one cut: the same values and bond as the all-library route."""
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of, to_dense_np
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(17)
    a = Leg((-1, 1, 3), (20, 90, 40), 1)
    b = Leg((-1, 1, 3), (25, 80, 45), -1)
    lay = layout_of((a, b), 0)
    h = rng.standard_normal(lay.size)
    h /= np.linalg.norm(h)
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    if method == "gram":
        lim = dict(LA._sytrd_table())
        monkeypatch.setitem(LA._SYTRD, "limits", {c: (min(v, 60) if v else 0) for c, v in lim.items()})
    else:
        lim = dict(LA._gebrd_table())
        monkeypatch.setitem(LA._GEBRD, "limits", {c: (min(v, 60) if v else 0) for c, v in lim.items()})
    U, S, V, d = LA.truncated_svd(m, 100, scale="right", method=method, host="device")
    U0, S0, V0, d0 = LA.truncated_svd(m, 100, scale="right", method=method, host="never")
    assert U.layout.legs == U0.layout.legs
    assert float((S - S0).abs().max()) <= 1e-12 * float(S0.max())
    dn = lambda t: to_dense_np(t.layout, t.data.cpu().numpy())
    assert np.abs(dn(U) @ dn(V) - dn(U0) @ dn(V0)).max() <= 1e-11


def test_rank_deficient_and_zero_sectors():
    """Exact zeros: a zero sector and a rank-1 sector on both device routes -- finite factors,
    the zero singular values, an orthonormal kept side."""
    from tnkit_gb300 import linalg as LA
    from tnkit_gb300.layout import Leg, layout_of, to_dense_np
    from tnkit_gb300.tensor import BlockTensor
    rng = np.random.default_rng(23)
    a = Leg((-1, 1, 3), (6, 30, 12), 1)
    b = Leg((-1, 1, 3), (5, 28, 14), -1)
    lay = layout_of((a, b), 0)
    h = np.zeros(lay.size)
    o = [int(x) for x in lay.offsets]
    h[o[1]:o[1] + 30 * 28] = np.outer(rng.standard_normal(30), rng.standard_normal(28)).ravel()
    h[o[2]:o[2] + 12 * 14] = rng.standard_normal(12 * 14) * 1e-3
    h /= np.linalg.norm(h)
    m = BlockTensor(lay, torch.as_tensor(h, device="cuda"), h)
    for method in ("gram", "svd"):
        U, S, V, d = LA.truncated_svd(m, 12, scale="right", method=method, host="device")
        U0, S0, V0, d0 = LA.truncated_svd(m, 12, scale="right", method=method, host="never")
        assert torch.isfinite(U.data).all() and torch.isfinite(V.data).all()
        assert torch.allclose(torch.sort(S).values, torch.sort(S0).values, rtol=0, atol=1e-10)
        Ud = to_dense_np(U.layout, U.data.cpu().numpy())
        assert np.abs(Ud.T @ Ud - np.eye(Ud.shape[1])).max() <= 1e-12
