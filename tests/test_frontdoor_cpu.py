"""The reference's own front doors (tnkit.dmrg, tnkit.tdvp2_evolve, tnkit.get_backend) with
backend='b200' installed, on a host without a GPU.

These tests import the reference package itself, so they run only where its checkout is
available (its path in the TNKIT_REF environment variable); elsewhere they are skipped. There is
no GPU here, so the GPU sweep is replaced by a recording stand-in: the tests check what reaches
this package (the reference's block tensors converted element for element, the options) and
what the reference's caller gets back (the reference's own tensor types, legs and numbers, the
reference's info keys), and that every other backend still runs the reference's own code.
The GPU side of the same path is tests/test_frontdoor_gpu.py."""
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

REF = os.environ.get("TNKIT_REF")
if not REF or not os.path.isdir(os.path.join(REF, "tnkit")):
    pytest.skip("the reference checkout is not available (set TNKIT_REF)", allow_module_level=True)


@pytest.fixture(scope="module")
def tnkit():
    sys.dont_write_bytecode = True
    if REF not in sys.path:
        sys.path.insert(0, REF)
    import tnkit as T
    from tnkit_gb300 import frontdoor
    frontdoor.install(T)
    yield T
    frontdoor.uninstall()


@pytest.fixture()
def on_cpu(monkeypatch):
    from tnkit_gb300 import frontdoor
    monkeypatch.setattr(frontdoor, "_device", lambda: torch.device("cpu"))


def _xxz_block(T, N):
    from tnkit_gb300 import workloads
    be = T.get_backend("numpy-real")
    return T.to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N, be, sym=T.U1())[0]


def test_get_backend_names_b200_everywhere(tnkit):
    from tnkit import _dmrg, backend, tdvp
    from tnkit_gb300.backend import B200Backend
    for mod in (tnkit, backend, _dmrg, tdvp):
        be = mod.get_backend("b200-real")
        assert isinstance(be, B200Backend) and be.dtype == torch.float64
    assert tnkit.get_backend("b200").dtype == torch.complex128
    assert tnkit.get_backend("b200-mixed").precision == "mixed"
    assert type(tnkit.get_backend("numpy-real")).__name__ == "NumpyBackend"


def test_dmrg_front_door_runs_the_gpu_sweep(tnkit, on_cpu, monkeypatch):
    """tnkit.dmrg(block MPO, backend='b200') hands the reference's MPO to this package's sweep
    (buffers identical to the reference's canonical ones) and returns the reference's types."""
    import importlib
    D = importlib.import_module("tnkit_gb300.dmrg")
    from tnkit_gb300.mpo import random_block_mps
    N, chi = 8, 6
    Wb = _xxz_block(tnkit, N)
    seen = {}

    def fake(W, c, **kw):
        seen.update(kw, W=W, chi=c)
        M = random_block_mps(W, c, kw["charge"], np.random.default_rng(kw["seed"]), device="cpu")
        info = {"sweeps": 1, "energies": [-3.0], "backend": "b200", "blocks": True,
                "eig": "lanczos-restart", "discarded_weight": 0.0, "matvec_calls": 7,
                "phase_time": {"eig": 0.0, "trunc": 0.0, "env": 0.0},
                "mixed_counts": {"lo": 0, "hi": 7}, "sites": 2, "expand": 0,
                "expand_alphas": [0.0], "sweep_s": [0.1], "precision": kw["precision"]}
        return -3.0, M, info
    monkeypatch.setattr(D, "dmrg", fake)
    E, mps, info = tnkit.dmrg(Wb, chi, backend="b200", charge=0, expand=0, seed=1, n_sweeps=3,
                              tol=0, rtol=0)
    assert E == -3.0 and seen["chi"] == chi and seen["charge"] == 0 and seen["seed"] == 1
    assert seen["n_sweeps"] == 3 and seen["precision"] == "f64" and seen["svd_method"] == "svd"
    for w_ref, w in zip(Wb, seen["W"]):
        c = w_ref.canonical()
        assert np.array_equal(np.asarray(c.data), w.data.numpy())
        assert [tuple(l.charges) for l in c.struct.legs] == [l.charges for l in w.legs]
    # the state comes back as the reference's block tensors, the reference's own random start
    from tnkit.block_backend import random_block_mps as ref_random
    ref0 = ref_random(Wb, chi, tnkit.get_backend("numpy-real"), 0, np.random.default_rng(1))
    assert type(mps).__name__ == "MPS" and mps.center == 0 and len(mps) == N
    for a, b in zip(mps, ref0):
        assert type(a).__name__ == "BlockTensor"
        assert a.struct is b.canonical().struct
        assert np.array_equal(a.data.numpy(), np.asarray(b.canonical().data))
    for key in ("sweeps", "energies", "backend", "blocks", "eig", "discarded_weight",
                "matvec_calls", "phase_time", "mixed_counts", "sites", "expand",
                "expand_alphas", "sweep_s"):
        assert key in info
    assert info["backend"] == "b200"


def test_dmrg_front_door_precision_specs(tnkit, on_cpu, monkeypatch):
    import importlib
    D = importlib.import_module("tnkit_gb300.dmrg")
    seen = {}
    monkeypatch.setattr(D, "dmrg", lambda W, c, **kw: (_ for _ in ()).throw(
        RuntimeError(kw["precision"] + "/" + kw["svd_method"])))
    Wb = _xxz_block(tnkit, 6)
    for spec, want in (("b200-mixed", "mixed/svd"), ("b200-ff", "ff/svd"),
                       ("b200-mixed-ff", "mixed-ff/svd")):
        with pytest.raises(RuntimeError, match=want):
            tnkit.dmrg(Wb, 4, backend=spec, charge=0, expand=0)
    with pytest.raises(RuntimeError, match="f64/gram"):
        tnkit.dmrg(Wb, 4, backend="b200", charge=0, expand=0, trunc="gram")
    from tnkit.block_backend import BlockBackend
    from tnkit_gb300.backend import B200Backend
    with pytest.raises(RuntimeError, match="mixed/svd"):
        tnkit.dmrg(Wb, 4, backend=BlockBackend(B200Backend(device="cpu", precision="mixed")),
                   charge=0, expand=0)


def test_dmrg_front_door_refuses_what_it_does_not_implement(tnkit, on_cpu):
    Wb = _xxz_block(tnkit, 6)
    with pytest.raises(NotImplementedError, match="expand=0"):
        tnkit.dmrg(Wb, 4, backend="b200", charge=0, n_sweeps=6)   # the block default expands
    with pytest.raises(NotImplementedError, match="sites"):
        tnkit.dmrg(Wb, 4, backend="b200", charge=0, expand=0, sites=1)
    with pytest.raises(NotImplementedError, match="reorth"):
        tnkit.dmrg(Wb, 4, backend="b200", charge=0, expand=0, reorth="none")
    with pytest.raises(NotImplementedError, match="eig"):
        tnkit.dmrg(Wb, 4, backend="b200", charge=0, expand=0, eig="lobpcg")


def test_dense_front_door_round_trip(tnkit, on_cpu, monkeypatch):
    import importlib
    from tnkit_gb300 import workloads
    D = importlib.import_module("tnkit_gb300.dmrg")
    from tnkit_gb300.mpo import random_dense_mps
    W = workloads.tfim_mpo(6, 1.0)
    seen = {}

    def fake(Wl, c, **kw):
        seen["W"] = Wl
        return -1.0, random_dense_mps(6, c, 2, np.random.default_rng(0), device="cpu"), {}
    monkeypatch.setattr(D, "dmrg", fake)
    E, mps, info = tnkit.dmrg(W, 4, backend="b200", n_sweeps=2)
    assert all(np.array_equal(a, b) for a, b in zip(seen["W"], W))
    shapes = [tuple(A.shape) for A in mps]
    assert shapes[0] == (1, 2, 2) and shapes[-1] == (2, 2, 1)
    assert all(isinstance(A, torch.Tensor) for A in mps)


def test_tdvp_front_door_runs_the_gpu_sweep(tnkit, on_cpu, monkeypatch):
    """tnkit.tdvp2_evolve(block MPS, backend='b200'): the state reaches this package's sweep as
    complex128 copies of the reference's buffers; `measure` sees the reference's tensors."""
    from tnkit_gb300 import tdvp as TD
    from tnkit.block_backend import random_block_mps as ref_random
    N = 6
    Wb = _xxz_block(tnkit, N)
    mps = [m.canonical() for m in ref_random(Wb, 4, tnkit.get_backend("numpy"), 0,
                                             np.random.default_rng(5))]
    seen = {}

    def fake(M, W, chi, dt, n, measure=None, **kw):
        seen.update(kw, M=M, chi=chi, dt=dt, n=n)
        rec = [(0.0, measure(M))] if measure is not None else []
        return M, rec
    monkeypatch.setattr(TD, "tdvp2_evolve", fake)
    kinds = []
    out, rec = tnkit.tdvp2_evolve(mps, Wb, 8, 0.05, 3, backend="b200",
                                  measure=lambda s: kinds.append(type(s[0]).__name__) or 1.0)
    assert seen["chi"] == 8 and seen["dt"] == 0.05 and seen["n"] == 3
    assert seen["krylov_m"] == 30 and seen["svd_method"] == "svd"
    for a, b in zip(seen["M"], mps):
        assert a.data.dtype == torch.complex128
        assert np.array_equal(a.data.numpy(), np.asarray(b.data).astype(complex))
    assert kinds == ["BlockTensor"] and rec == [(0.0, 1.0)]
    assert out.center == 0 and type(out[0]).__name__ == "BlockTensor"
    with pytest.raises(NotImplementedError, match="svd_tol"):
        tnkit.tdvp2_evolve(mps, Wb, 8, 0.05, 1, backend="b200", svd_tol=1e-8)


def test_other_backends_still_run_the_reference(tnkit):
    from tnkit_gb300 import workloads
    W = [np.real(w) for w in workloads.tfim_mpo(6, 1.0)]
    E1, _, info = tnkit.dmrg(W, 8, n_sweeps=3, tol=0, rtol=0, seed=0, backend="numpy-real")
    from tnkit_gb300 import frontdoor
    frontdoor.uninstall()
    try:
        E0, _, _ = tnkit.dmrg(W, 8, n_sweeps=3, tol=0, rtol=0, seed=0, backend="numpy-real")
    finally:
        frontdoor.install(tnkit)
    assert E1 == E0 and info["backend"] == "numpy-real"
