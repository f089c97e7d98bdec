"""The backend adaptor's surface on a host without a GPU: names, the reference's interface
methods, and its error behaviour (no CPU fallback for the hot path)."""
import numpy as np
import pytest


def test_get_backend_names():
    from tnkit_gb300.backend import B200Backend, get_backend
    be = get_backend("b200")
    assert isinstance(be, B200Backend) and be.name == "b200" and be.is_torch
    assert get_backend("b200-mixed").precision == "mixed"
    assert get_backend(be) is be
    with pytest.raises(ValueError):
        get_backend("numpy")


def test_interface_methods_present():
    from tnkit_gb300.backend import B200Backend
    for name in ("einsum", "array", "to_numpy", "randn", "zeros", "ones", "zeros_like", "conj",
                 "transpose", "diag", "vdot", "norm", "to_scalar", "svd", "qr", "eigh",
                 "astype", "sync", "apply_two_site", "apply_one_site", "update_left_env",
                 "update_right_env", "tensordot", "dmrg"):
        assert callable(getattr(B200Backend, name)), name


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
