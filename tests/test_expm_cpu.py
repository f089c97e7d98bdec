"""exp(tau T) e_1 of a real symmetric tridiagonal T by its eigendecomposition (the Krylov
exponential's default route) against scipy's Pade expm of the full matrix (the reference's
per-iteration host call), for imaginary (TDVP) and real tau, j = 1 .. 30."""
import numpy as np
import pytest

from tnkit_gb300.expm import _expm_col


@pytest.mark.parametrize("j", [1, 2, 5, 12, 30])
@pytest.mark.parametrize("tau", [-0.05j, -0.5j, 0.3, -1.0 + 0.2j])
def test_eigh_route_matches_pade(j, tau):
    rng = np.random.default_rng(j)
    a = list(rng.standard_normal(j) * 3.0)
    b = list(np.abs(rng.standard_normal(j)))
    x = _expm_col(tau, a, b, "eigh")
    y = _expm_col(tau, a, b, "pade")
    assert np.abs(x - y).max() <= 1e-13 * max(1.0, np.abs(y).max())


def test_route_name_checked():
    with pytest.raises(ValueError):
        _expm_col(-0.1j, [1.0, 2.0], [0.5], "taylor")
