"""tnk_apply_two_site_f64_noalloc: the two-site matvec for callers that cannot allocate device
memory (host callbacks, fixed memory pools, bindings without a device allocator). It uses the
library's fixed scratch array instead of a caller workspace.

Checked through the C ABI against tnk_apply_two_site_f64 (which takes a caller workspace) on two
calls in a row with different problems, so the second call cannot pass on what the first left in
the shared scratch. Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build, _lib
    build.build()
    return _lib.load()


def _problem(scale, seed):
    from tnkit_gb300 import ops, workloads
    dims = [max(1, d // scale) for d in workloads.C2_MID_DIMS]
    th, L, W1, W2, R = workloads.mid_bond_problem(dims=dims, seed=seed)
    return ops.TwoSiteOperator(th.layout, L, W1, W2, R), th


def test_noalloc_matches_workspace_entry_point_twice(lib):
    from tnkit_gb300 import _lib
    cap = C.c_int64()
    assert lib.tnk_noalloc_scratch_elems(C.byref(cap)) == 0
    stream = _lib.stream_ptr()
    for scale, seed in ((4, 11), (1, 12)):          # a small problem, then the chi=1024 one
        op, th = _problem(scale, seed)
        p = op.plan
        assert p.ws_elems <= cap.value
        x = th.data
        ref = torch.empty_like(x)
        ws = torch.empty(p.ws_elems, dtype=torch.float64, device=x.device)
        _lib.check(lib.tnk_apply_two_site_f64(C.byref(p.c), op.L.data.data_ptr(), x.data_ptr(),
                                              op.R.data.data_ptr(), ref.data_ptr(),
                                              ws.data_ptr(), ws.numel(), stream), "ws")
        got = torch.full_like(x, float("nan"))
        _lib.check(lib.tnk_apply_two_site_f64_noalloc(C.byref(p.c), op.L.data.data_ptr(),
                                                      x.data_ptr(), op.R.data.data_ptr(),
                                                      got.data_ptr(), stream), "noalloc")
        torch.cuda.synchronize()
        err = float((got - ref).abs().max() / ref.abs().max())
        assert np.isfinite(err) and err <= TOL, (scale, err)


def test_noalloc_rejects_plans_beyond_the_scratch(lib):
    """A plan needing more scratch than the fixed array is refused on the host, before any
    launch, with TNK_ERR_SIZE and a message naming the limit."""
    from tnkit_gb300 import _lib
    op, th = _problem(4, 13)
    big = _lib.Plan3.from_buffer_copy(op.plan.c)
    cap = C.c_int64()
    lib.tnk_noalloc_scratch_elems(C.byref(cap))
    big.ws1_elems = cap.value
    big.ws2_elems = 1
    out = torch.empty_like(th.data)
    rc = lib.tnk_apply_two_site_f64_noalloc(C.byref(big), op.L.data.data_ptr(),
                                            th.data.data_ptr(), op.R.data.data_ptr(),
                                            out.data_ptr(), _lib.stream_ptr())
    assert rc == _lib.TNK_ERR_SIZE
    assert b"TNK_NOALLOC_SCRATCH_ELEMS" in lib.tnk_last_error()
