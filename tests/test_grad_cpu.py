"""The gradient machinery's tables on the CPU (table interpreter, no GPU): the reversed
environment is the dense transpose element for element, the transposed two-site operator is the
adjoint (<g, H theta> = <H^T g, theta>), and a bond operator applied with identity environments
is the two-site operator on theta's physical legs."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from table_interp import run_comb, run_plan3


def _problem(seed):
    from tnkit_gb300 import workloads
    return workloads.mid_bond_problem(dims=(1, 3, 5, 4, 2), charges=(-4, -2, 0, 2, 4),
                                      seed=seed, device="cpu")


def test_reversed_environment_is_the_transpose():
    from tnkit_gb300 import grad
    from tnkit_gb300.layout import from_dense_np, to_dense_np
    th, L, W1, W2, R = _problem(1)
    for E in (L, R):
        hp = grad._plan_reverse3(E.layout)
        out = np.full(hp.out_layout.size, np.nan)
        run_comb(hp.c, E.host, out)
        want = from_dense_np(hp.out_layout, to_dense_np(E.layout, E.host).transpose(2, 1, 0))
        assert np.array_equal(out, want)


def test_transposed_operator_is_the_adjoint():
    from tnkit_gb300 import grad, plan as P
    from tnkit_gb300.layout import from_dense_np, to_dense_np
    from tnkit_gb300.ops import _host_of
    from tnkit_gb300.tensor import BlockTensor
    th, L, W1, W2, R = _problem(2)

    def rev(E):
        hp = grad._plan_reverse3(E.layout)
        out = np.zeros(hp.out_layout.size)
        run_comb(hp.c, E.host, out)
        return BlockTensor(hp.out_layout, torch.as_tensor(out), out)
    Lt, Rt = rev(L), rev(R)
    W1t, W2t = grad.transpose_mpo(W1), grad.transpose_mpo(W2)
    fwd = P.plan_apply(th.layout, L.layout, [(W1.layout, _host_of(W1)),
                                             (W2.layout, _host_of(W2))], R.layout)
    adj = P.plan_apply(th.layout, Lt.layout, [(W1t.layout, _host_of(W1t)),
                                              (W2t.layout, _host_of(W2t))], Rt.layout)
    assert adj.out_layout.size == th.layout.size
    rng = np.random.default_rng(3)
    x, g = rng.standard_normal(th.layout.size), rng.standard_normal(th.layout.size)
    hx = run_plan3(fwd, L.host, x, R.host)
    htg = run_plan3(adj, Lt.host, g, Rt.host)
    a, b = float(g @ hx), float(htg @ x)
    assert abs(a - b) <= 1e-13 * (np.abs(g) @ np.abs(hx) + 1.0)


def test_bond_operator_with_identity_environments():
    from tnkit_gb300 import grad, plan as P
    from tnkit_gb300.layout import to_dense_np
    from tnkit_gb300.mpo import to_block_mpo
    from tnkit_gb300.ops import _host_of
    th, *_ = _problem(4)
    W1, W2 = to_block_mpo(grad.xxz_bond_operator(0.7), [[1, -1]] * 2, device="cpu")[0]
    L = grad._identity_env(th.legs[0], W1.legs[0].flip(), "cpu")
    R = grad._identity_env(th.legs[3], W2.legs[1].flip(), "cpu")
    hp = P.plan_apply(th.layout, L.layout, [(W1.layout, _host_of(W1)),
                                            (W2.layout, _host_of(W2))], R.layout)
    y = run_plan3(hp, L.host, th.host, R.host)
    # dense: h on the physical legs (basis up, down: the sector order of charges -1, +1)
    sp = np.array([[0.0, 0.0], [1.0, 0.0]])          # S+ in the (down, up) sector order
    sm, sz = sp.T.copy(), np.diag([-0.5, 0.5])
    h = 0.5 * (np.kron(sp, sm) + np.kron(sm, sp)) + 0.7 * np.kron(sz, sz)
    t = to_dense_np(th.layout, th.host)
    a, d = t.shape[0], t.shape[3]
    want = np.einsum("xy,ayb->axb", h, t.reshape(a, 4, d)).reshape(t.shape)
    got = to_dense_np(hp.out_layout, y)
    assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()
