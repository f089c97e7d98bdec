"""The batched operator (tnkit_gb300.batch.BatchedTwoSiteOperator) on the GPU: one set of
launches for many chains' local problems gives each problem's own FP64 matvec (only the split-K
summation order differs), the float-float variant stays within FP64-grade accuracy, the
tensor-core variant (split TF32) within 2e-5, and a CUDA graph capture of the batched call
replays it exactly."""
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


@pytest.fixture(scope="module")
def problems():
    from tnkit_gb300 import batch as B
    return B.batch_problems(24, seed=2)


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("precision,tol", [("f64", 1e-13), ("ff", 1e-12), ("tc", 2e-5)])
def test_batched_matches_each_problem(problems, precision, tol):
    from tnkit_gb300 import batch as B, ops
    op = B.BatchedTwoSiteOperator(problems, precision=precision)
    x = torch.randn(op.n, dtype=torch.float64, device="cuda")
    y = op(x)
    if op.tc is not None:
        op.tc.check_device_error()
    for xk, yk, (th, L, W1, W2, R) in zip(op.split(x), op.split(y), problems):
        ref = ops.TwoSiteOperator(th, L, W1, W2, R)(xk.contiguous())
        assert _rel(yk, ref) <= tol


def test_batched_graph_replay_is_exact(problems):
    from tnkit_gb300 import batch as B
    op = B.BatchedTwoSiteOperator(problems)
    x = torch.randn(op.n, dtype=torch.float64, device="cuda")
    y, yg = torch.empty_like(x), torch.empty_like(x)
    op(x, y)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        op(x, yg)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, yg)
    x.copy_(torch.randn_like(x))        # the graph reads the buffer's current contents
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(op(x), yg)


def test_batched_rejects_wrong_length(problems):
    from tnkit_gb300 import batch as B
    op = B.BatchedTwoSiteOperator(problems[:3])
    with pytest.raises(ValueError):
        op(torch.zeros(op.n + 1, dtype=torch.float64, device="cuda"))


def test_set_active_skips_only_the_masked_problems(problems):
    """Dropping problems' launch grids leaves the others' results bit-identical and the
    dropped problems' output untouched; restoring the mask restores the full result."""
    from tnkit_gb300 import batch as B
    op = B.BatchedTwoSiteOperator(problems[:10])
    x = torch.randn(op.n, dtype=torch.float64, device="cuda")
    full = op(x)
    mask = np.array([k % 3 != 1 for k in range(10)])
    op.set_active(mask)
    y = torch.full_like(x, 7.0)
    op(x, y)
    for k, (a, b) in enumerate(zip(op.split(y), op.split(full))):
        if mask[k]:
            assert torch.equal(a, b), k
        else:
            assert bool((a == 7.0).all()), k
    op.set_active(np.ones(10, bool))
    assert torch.equal(op(x), full)
