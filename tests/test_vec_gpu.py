"""The Lanczos vector kernels through the C ABI against numpy float64: the fused Gram-Schmidt
pass (tnk_cgs_pass_f64) in every mode, across the row-count boundaries of its launch shapes
(16 / 32 / 64 rows), ragged and empty vectors, and the older multi-dot / GEMV entry points that
now share its kernels. Reductions run in a different order from numpy's, so the bar is a
relative 1e-13 of the magnitudes summed."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SUB, DOT, NRM = 1, 2, 4


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


class _Ctx:
    def __init__(self):
        from tnkit_gb300 import _lib
        self.lib = _lib.lib()
        self.lib_mod = _lib
        self.red = torch.empty(_lib.TNK_RED_ELEMS, dtype=torch.float64, device="cuda")
        self.cnt = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.sp = _lib.stream_ptr()

    def cgs(self, V, nv, cin, w, out, mode):
        rc = self.lib.tnk_cgs_pass_f64(V.data_ptr(), V.stride(0), nv,
                                       None if cin is None else cin.data_ptr(), w.data_ptr(),
                                       w.numel(), None if out is None else out.data_ptr(), mode,
                                       self.red.data_ptr(), self.cnt.data_ptr(), self.sp)
        return rc


@pytest.fixture(scope="module")
def ctx():
    return _Ctx()


def _data(nv, n, ld, seed):
    rng = np.random.default_rng(seed)
    V = rng.standard_normal((max(nv, 1), ld))
    w = rng.standard_normal(n) * 3.0
    c = rng.standard_normal(max(nv, 1))
    return V, w, c


@pytest.mark.parametrize("nv", [1, 7, 16, 17, 32, 33, 41, 64])
@pytest.mark.parametrize("n,ld", [(1, 1), (1000, 1003), (808598, 808598)])
def test_cgs_modes_match_numpy(ctx, nv, n, ld):
    V, w, c = _data(nv, n, ld, nv * 7 + n)
    Vd = torch.as_tensor(V, device="cuda")
    cd = torch.as_tensor(c, device="cuda")
    Vn = V[:nv, :n]
    scale_dot = np.abs(Vn) @ np.abs(w)
    # DOT
    wd = torch.as_tensor(w, device="cuda")
    out = torch.full((66,), np.nan, dtype=torch.float64, device="cuda")
    assert ctx.cgs(Vd, nv, None, wd, out, DOT) == 0
    got = out[:nv].cpu().numpy()
    assert np.all(np.abs(got - Vn @ w) <= 1e-13 * scale_dot + 1e-300)
    assert np.isnan(out[nv].item()) or nv == 64
    # SUB | DOT
    ws = w - c[:nv] @ Vn
    assert ctx.cgs(Vd, nv, cd, wd, out, SUB | DOT) == 0
    sub_scale = np.abs(w) + np.abs(c[:nv]) @ np.abs(Vn)
    assert np.all(np.abs(wd.cpu().numpy() - ws) <= 1e-14 * sub_scale)
    assert np.all(np.abs(out[:nv].cpu().numpy() - Vn @ ws)
                  <= 1e-13 * (np.abs(Vn) @ sub_scale) + 1e-300)
    # SUB | NRM
    wd = torch.as_tensor(w, device="cuda")
    assert ctx.cgs(Vd, nv, cd, wd, out, SUB | NRM) == 0
    assert abs(out[0].item() - np.linalg.norm(ws)) <= 1e-13 * np.linalg.norm(sub_scale)
    # SUB alone
    wd = torch.as_tensor(w, device="cuda")
    assert ctx.cgs(Vd, nv, cd, wd, None, SUB) == 0
    assert np.all(np.abs(wd.cpu().numpy() - ws) <= 1e-14 * sub_scale)
    # the completion counter is left zero
    assert int(ctx.cnt.abs().sum().item()) == 0


def test_cgs_norm_only_and_empty(ctx):
    w = torch.as_tensor(np.arange(1.0, 11.0), device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    assert ctx.cgs(w.view(1, -1), 0, None, w, out, NRM) == 0
    assert abs(out[0].item() - np.linalg.norm(np.arange(1.0, 11.0))) <= 1e-14 * 20
    e = torch.zeros(0, dtype=torch.float64, device="cuda")
    V = torch.zeros((3, 0), dtype=torch.float64, device="cuda")
    out = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
    assert ctx.cgs(V, 3, None, e, out, DOT) == 0
    assert out[:3].abs().sum().item() == 0.0
    assert ctx.cgs(V, 3, out, e, out, SUB | NRM) == 0
    assert out[0].item() == 0.0


def test_cgs_rejects_bad_arguments(ctx):
    w = torch.zeros(8, dtype=torch.float64, device="cuda")
    V = torch.zeros((65, 8), dtype=torch.float64, device="cuda")
    out = torch.zeros(70, dtype=torch.float64, device="cuda")
    E = ctx.lib_mod.TNK_ERR_ARG
    assert ctx.cgs(V, 65, None, w, out, DOT) == E           # more than 64 rows
    assert ctx.cgs(V, 4, None, w, out, DOT | NRM) == E      # exclusive modes
    assert ctx.cgs(V, 4, None, w, out, SUB) == E            # subtraction without coefficients
    assert ctx.cgs(V, 4, None, w, out, 0) == E
    assert ctx.cgs(V, 4, None, w, out, 8) == E


@pytest.mark.parametrize("nv", [5, 40])
def test_multidot_and_gemv_sub_entry_points(ctx, nv):
    n = 100003
    V, w, c = _data(nv, n, n, 11 + nv)
    Vd, wd = torch.as_tensor(V, device="cuda"), torch.as_tensor(w, device="cuda")
    out = torch.zeros(64, dtype=torch.float64, device="cuda")
    lib = ctx.lib
    assert lib.tnk_multidot_f64(Vd.data_ptr(), n, nv, wd.data_ptr(), n, out.data_ptr(),
                                ctx.red.data_ptr(), ctx.sp) == 0
    assert np.all(np.abs(out[:nv].cpu().numpy() - V @ w) <= 1e-13 * (np.abs(V) @ np.abs(w)))
    cd = torch.as_tensor(c, device="cuda")
    assert lib.tnk_gemv_sub_f64(Vd.data_ptr(), n, nv, cd.data_ptr(), wd.data_ptr(), n,
                                ctx.sp) == 0
    ws = w - c @ V
    assert np.all(np.abs(wd.cpu().numpy() - ws) <= 1e-14 * (np.abs(w) + np.abs(c) @ np.abs(V)))


def test_pipelined_lanczos_without_speculation_agrees():
    """The queued-ahead loop and the wait-every-iteration loop give the same eigenpair and
    iteration count on a matrix whose solve restarts."""
    from tnkit_gb300.lanczos import lanczos_ground_restart
    rng = np.random.default_rng(5)
    n = 500
    A = rng.standard_normal((n, n))
    H = torch.as_tensor((A + A.T) / 2, device="cuda")
    v0 = torch.as_tensor(rng.standard_normal(n), device="cuda")
    mv = lambda v, out: out.copy_(H @ v)
    e1, x1, i1 = lanczos_ground_restart(mv, v0, tol=1e-10, max_iter=400, m=20, k=6)
    e2, x2, i2 = lanczos_ground_restart(mv, v0, tol=1e-10, max_iter=400, m=20, k=6,
                                        speculate=False)
    ev = np.linalg.eigvalsh((A + A.T) / 2)[0]
    assert i1["restarts"] > 0 and i1["converged"] and i2["converged"]
    assert i1["iters"] == i2["iters"] and i2["discarded"] == 0 and i1["discarded"] <= 1
    assert abs(e1 - ev) <= 1e-10 * abs(ev) and abs(e2 - ev) <= 1e-10 * abs(ev)
    assert abs(abs(float(torch.dot(x1, x2))) - 1.0) <= 1e-9


@pytest.mark.parametrize("nv", [1, 16, 33])
def test_cgs_f32_modes_match_numpy(ctx, nv):
    """The FP32 pass: FP32 arithmetic, so the bar is FP32 rounding of the summed magnitudes."""
    n = 200003
    V, w, c = _data(nv, n, n, 100 + nv)
    V32, w32 = V.astype(np.float32), w.astype(np.float32)
    Vd = torch.as_tensor(V32, device="cuda")
    cd = torch.as_tensor(c, device="cuda")
    lib = ctx.lib
    out = torch.zeros(66, dtype=torch.float64, device="cuda")

    def run(wd, mode, cin=None):
        return lib.tnk_cgs_pass_f32(Vd.data_ptr(), n, nv,
                                    None if cin is None else cin.data_ptr(), wd.data_ptr(), n,
                                    out.data_ptr(), mode, ctx.red.data_ptr(),
                                    ctx.cnt.data_ptr(), ctx.sp)
    Vn, wn = V32[:nv].astype(np.float64), w32.astype(np.float64)
    wd = torch.as_tensor(w32, device="cuda")
    assert run(wd, DOT) == 0
    tol = 4e-6 * (np.abs(Vn) @ np.abs(wn))
    assert np.all(np.abs(out[:nv].cpu().numpy() - Vn @ wn) <= tol)
    ws = wn - c[:nv] @ Vn
    assert run(wd, SUB | NRM, cd) == 0
    scale = np.abs(wn) + np.abs(c[:nv]) @ np.abs(Vn)
    # one FP32 rounding per row of the FMA chains (and of the coefficients)
    assert np.all(np.abs(wd.cpu().numpy() - ws) <= (nv + 2) * 1.2e-7 * scale)
    assert abs(out[0].item() - np.linalg.norm(ws)) <= (nv + 2) * 1.2e-7 * np.linalg.norm(scale)
    assert int(ctx.cnt.abs().sum().item()) == 0


def test_lanczos_fp32_basis_matches_eigvalsh():
    """The FP32-basis Lanczos (tensor-core stage of the mixed solve) reaches FP32-level accuracy
    and restarts like the FP64 one."""
    from tnkit_gb300.lanczos import lanczos_ground_restart
    rng = np.random.default_rng(8)
    n = 600
    A = rng.standard_normal((n, n))
    A = (A + A.T) / 2
    H32 = torch.as_tensor(A, dtype=torch.float32, device="cuda")
    v0 = torch.as_tensor(rng.standard_normal(n), device="cuda")
    mv = lambda v, out: torch.mv(H32, v, out=out)
    e, x, info = lanczos_ground_restart(mv, v0, tol=1e-4, max_iter=600, m=30, k=8,
                                        dtype=torch.float32)
    ev, evec = np.linalg.eigh(A)
    assert x.dtype == torch.float32 and info["converged"] and info["restarts"] > 0
    assert abs(e - ev[0]) <= 1e-5 * abs(ev[0])
    assert abs(abs(float(np.dot(x.double().cpu().numpy(), evec[:, 0]))) - 1.0) <= 1e-4


@pytest.mark.parametrize("nv,kk,n,ld", [(40, 10, 808598, 808598), (64, 64, 1003, 1010),
                                        (17, 33, 200003, 200003), (1, 1, 1, 1), (5, 3, 0, 0),
                                        (0, 4, 100, 100)])
def test_rotate_f32_matches_numpy(ctx, nv, kk, n, ld):
    """The thick-restart rotation of an FP32 basis (tnk_rotate_f32): out = Y^T V[:nv], FP32
    FMA chains in ascending row order, coefficients rounded to FP32 -- bar (nv + 2) FP32
    roundings of the summed magnitudes; nv = 0 writes zeros."""
    rng = np.random.default_rng(nv * 31 + kk + n)
    V = rng.standard_normal((max(nv, 1), max(ld, 1))).astype(np.float32)
    Y = rng.standard_normal((max(nv, 1), kk))
    Vd = torch.as_tensor(V, device="cuda")
    Yd = torch.as_tensor(Y[:nv].copy() if nv else Y, device="cuda")
    out = torch.full((kk, max(ld, 1)), 7.0, dtype=torch.float32, device="cuda")
    rc = ctx.lib.tnk_rotate_f32(Vd.data_ptr(), max(ld, 1), nv, Yd.data_ptr(), kk, out.data_ptr(),
                                max(ld, 1), n, ctx.sp)
    assert rc == 0
    got = out[:, :n].double().cpu().numpy()
    Vn = V[:nv, :n].astype(np.float64)
    want = Y[:nv].T @ Vn
    scale = np.abs(Y[:nv]).T @ np.abs(Vn)
    assert np.all(np.abs(got - want) <= (nv + 2) * 1.2e-7 * scale + 1e-30)
    if ld > n:                                       # columns past n untouched
        assert bool((out[:, n:] == 7.0).all())


def test_rotate_f32_rejects_bad_arguments(ctx):
    V = torch.zeros((2, 8), dtype=torch.float32, device="cuda")
    Y = torch.zeros((2, 2), dtype=torch.float64, device="cuda")
    out = torch.zeros((2, 8), dtype=torch.float32, device="cuda")
    lib = ctx.lib
    args = lambda nv, kk, ldv, ldo, n: (V.data_ptr(), ldv, nv, Y.data_ptr(), kk, out.data_ptr(),
                                       ldo, n, ctx.sp)
    assert lib.tnk_rotate_f32(*args(65, 2, 8, 8, 8)) != 0       # nv above 64
    assert lib.tnk_rotate_f32(*args(2, 0, 8, 8, 8)) != 0        # no kept vectors
    assert lib.tnk_rotate_f32(*args(2, 65, 8, 8, 8)) != 0       # kk above 64
    assert lib.tnk_rotate_f32(*args(2, 2, 4, 8, 8)) != 0        # ldv < n
    assert lib.tnk_rotate_f32(*args(2, 2, 8, 4, 8)) != 0        # ldo < n
    assert lib.tnk_rotate_f32(*args(2, 2, 8, 8, -1)) != 0       # negative length
