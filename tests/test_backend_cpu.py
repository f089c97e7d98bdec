"""The backend adaptor's surface on a host without a GPU: names, the reference's interface
methods, and its error behaviour (no CPU fallback for the hot path)."""
import numpy as np
import pytest


def test_get_backend_names():
    """'b200' is complex128 and 'b200-real' float64, as the reference's 'torch-cuda' and
    'torch-cuda-real' (tnkit/backend.py:192-240); the float-float and mixed specs are real."""
    import torch
    from tnkit_gb300.backend import B200Backend, get_backend
    be = get_backend("b200", device="cpu")
    assert isinstance(be, B200Backend) and be.name == "b200" and be.is_torch
    assert be.is_complex and be.dtype == torch.complex128 and be.rdtype == torch.float64
    real = get_backend("b200-real", device="cpu")
    assert not real.is_complex and real.dtype == torch.float64 and real.name == "b200-real"
    assert get_backend("b200-mixed").precision == "mixed"
    assert get_backend("b200-mixed-ff").precision == "mixed-ff"
    assert get_backend("b200-ff").precision == "ff"
    assert get_backend(be) is be
    with pytest.raises(ValueError):
        get_backend("numpy")


def test_interface_methods_present():
    from tnkit_gb300.backend import B200Backend
    # every method of the reference's backend interface (tnkit/backend.py:491-816) ...
    for name in ("einsum", "array", "to_numpy", "randn", "zeros", "ones", "zeros_like", "conj",
                 "transpose", "diag", "vdot", "norm", "to_scalar", "svd", "svd_batched", "qr",
                 "eigh", "astype", "stack", "tridiag", "expm", "expm_host",
                 "expm_sym_tridiag_eigh", "expm_sym_tridiag_eigh_batched", "expm_taylor", "mv",
                 "vm", "guard_denom", "norm_axis", "stack_axis", "sync"):
        assert callable(getattr(B200Backend, name)), name
    # ... and the hot path on block tensors
    for name in ("apply_two_site", "apply_one_site", "update_left_env", "update_right_env",
                 "tensordot", "truncated_svd", "dmrg", "tdvp2_evolve"):
        assert callable(getattr(B200Backend, name)), name


def test_dense_interface_semantics_on_the_host():
    """The small dense helpers behave as the reference's TorchBackend's (on CPU tensors here;
    the GPU runs the same torch calls)."""
    import torch
    from scipy.linalg import expm
    from tnkit_gb300.backend import B200Backend
    be = B200Backend(device="cpu", complex=True)
    rng = np.random.default_rng(0)
    d = torch.as_tensor(rng.standard_normal(5))
    e = torch.as_tensor(rng.standard_normal(4))
    T = be.tridiag(d, e)
    assert T.dtype == torch.complex128
    Tn = np.diag(d.numpy()) + np.diag(e.numpy(), 1) + np.diag(e.numpy(), -1)
    assert np.allclose(T.numpy(), Tn)
    assert np.allclose(be.expm(0.1j * T).numpy(), expm(0.1j * Tn))
    assert np.allclose(be.expm_host(0.1j * T), expm(0.1j * Tn))
    assert np.allclose(be.expm_taylor(0.1j * T, 4).numpy(), expm(0.1j * Tn), atol=1e-13)
    x = torch.as_tensor(rng.standard_normal(5) + 0j)
    assert torch.allclose(be.mv(T, x), T @ x) and torch.allclose(be.vm(x, T), x @ T)
    g = be.guard_denom(torch.tensor([0.0, 1e-300, 2.0], dtype=torch.float64))
    assert g.tolist() == [1e-200, 1e-200, 2.0]
    st = be.stack([torch.tensor(1.0), 2.0])
    assert st.tolist() == [1.0, 2.0]
    xs = [torch.ones(3), 2 * torch.ones(3)]
    assert be.stack_axis(xs, 0).shape == (2, 3)
    assert torch.allclose(be.norm_axis(torch.ones(2, 4), -1), torch.full((2,), 2.0))
    assert be.astype(torch.ones(2), "low").dtype == torch.complex64
    real = B200Backend(device="cpu")
    assert real.astype(torch.ones(2), "low").dtype == torch.float32
    assert real.randn(np.random.default_rng(1), (3,)).dtype == torch.float64
    assert be.randn(np.random.default_rng(1), (3,)).dtype == torch.complex128


def test_hot_path_refuses_host_tensors():
    """Block tensors on the host are refused, not computed on the CPU."""
    import torch
    from tnkit_gb300 import workloads, ops
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=[1, 2, 1], charges=[-2, 0, 2],
                                                  device="cpu")
    with pytest.raises(TypeError):
        ops.apply_two_site(th, L, W1, W2, R)


def test_real_backend_rejects_imaginary_parts():
    import torch
    from tnkit_gb300.backend import B200Backend
    be = B200Backend(device="cpu")
    assert be.array(np.ones(3)).dtype == torch.float64
    with pytest.raises(TypeError):
        be.array(np.array([1.0 + 1.0j]))
