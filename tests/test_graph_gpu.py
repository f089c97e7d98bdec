"""CUDA-graph replay of the local matvec (ops.GraphedOperator, the counterpart of the
reference's MatvecGraph, tnkit/block_graph.py:124-180): after one eager call the launch
sequence replays from a graph and gives bit-identical results; a DMRG run with graph=True
reproduces the eager run's energies exactly."""
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


@pytest.mark.parametrize("precision", ["f64", "ff"])
def test_graphed_matvec_is_bit_identical(precision):
    from tnkit_gb300 import ops, workloads
    dims = [max(1, d // 4) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=7)
    eager = ops.TwoSiteOperator(th.layout, L, W1, W2, R, precision=precision)
    g = ops.GraphedOperator(ops.TwoSiteOperator(th.layout, L, W1, W2, R, precision=precision),
                            th.layout.size)
    w = torch.empty_like(th.data)
    for k in range(4):
        x = torch.randn_like(th.data)
        ref = eager(x)
        got = g(x, w) if k % 2 else g(x)
        torch.cuda.synchronize()
        assert torch.equal(got, ref), k
    assert g.eager == 1 and g.replays == 3 and g.calls == 4


def test_dmrg_with_graphs_matches_eager():
    from tnkit_gb300 import workloads
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.mpo import to_block_mpo
    Wb = lambda: to_block_mpo(workloads.xxz_mpo(16), [[1, -1]] * 16)[0]
    kw = dict(charge=0, seed=1, n_sweeps=3, tol=0, rtol=0, expand=0)
    E0, _, i0 = dmrg(Wb(), 32, **kw)
    E1, _, i1 = dmrg(Wb(), 32, graph=True, **kw)
    assert i1["energies"] == i0["energies"] and E1 == E0
