"""The conversion the reference's front door uses, on the GPU: tensors shaped like the
reference's `tnkit.blocks.BlockTensor` (a `struct` with legs and charge, `canonical()`, a flat
host buffer) go through `BlockTensor.from_reference` into the kernels and the GPU sweep, and give
the reference's own results (tests/golden). The reference package is not importable where the
GPU runs, so its tensors are stood in for by objects with the same attributes; the routing of
the reference's `dmrg` / `tdvp2_evolve` / `get_backend` to this package is
tests/test_frontdoor_cpu.py."""
import json
import os
from types import SimpleNamespace

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import GOLDEN


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tnkit_gb300 import build
    build.build()


class RefShaped:
    """The attributes of a reference BlockTensor that the conversion reads."""
    is_block = True

    def __init__(self, legs, charge, data):
        self.struct = SimpleNamespace(
            legs=tuple(SimpleNamespace(charges=tuple(l["charges"]), dims=tuple(l["dims"]),
                                       sign=l["sign"]) for l in legs), charge=charge)
        self.data = np.asarray(data)

    def canonical(self):
        return self


def _ref_shaped(t):
    legs = [{"charges": l.charges, "dims": l.dims, "sign": l.sign} for l in t.layout.legs]
    return RefShaped(legs, t.layout.charge, t.data.detach().cpu().numpy())


def test_from_reference_two_site_matches_reference_golden(golden):
    from tnkit_gb300 import BlockTensor, ops
    meta, A = golden
    tag = "xxz12_b5"
    ts = [BlockTensor.from_reference(RefShaped(meta[f"{tag}_{k}"]["legs"],
                                               meta[f"{tag}_{k}"]["charge"], A[f"{tag}_{k}"]))
          for k in ("theta", "L", "W1", "W2", "R")]
    assert all(t.data.is_cuda and t.data.dtype == torch.float64 for t in ts)
    out = ops.apply_two_site(*ts).data.cpu().numpy()
    ref = A[f"{tag}_H2theta"]
    assert np.abs(out - ref).max() <= 1e-13 * np.abs(ref).max()


def test_from_reference_complex_state_stays_complex(golden):
    from tnkit_gb300 import BlockTensor
    meta, A = golden
    x = A["xxz12_b5_theta"] * (1.0 + 0.5j)
    t = BlockTensor.from_reference(RefShaped(meta["xxz12_b5_theta"]["legs"], 0, x))
    assert t.data.dtype == torch.complex128 and t.host is None
    assert np.array_equal(t.data.cpu().numpy(), x)


def test_block_dmrg_through_the_conversion_matches_reference():
    """The block MPO as the reference's to_block_mpo lays it out (canonical buffers), converted
    as the front door converts it, runs the sweep to the reference's every-sweep energies."""
    from tnkit_gb300 import BlockTensor, workloads
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.mpo import to_block_mpo
    ref = json.load(open(os.path.join(GOLDEN, "dmrg_small.json")))["xxz_n12_chi16"]
    W = to_block_mpo(workloads.xxz_mpo(12), [[1, -1]] * 12, device="cpu")[0]
    Wc = [BlockTensor.from_reference(_ref_shaped(w)) for w in W]
    E, M, info = dmrg(Wc, 16, charge=0, seed=1, n_sweeps=4, tol=0, rtol=0, expand=0)
    assert np.allclose(info["energies"], ref["energies"], rtol=1e-12, atol=0)
    assert abs(info["discarded_weight"] - ref["discarded_weight"]) <= 1e-12
