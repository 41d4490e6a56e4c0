"""CPU: the LXEB reference value against the reference's own piquasso/lxeb.py
(tests/golden/lxeb_values.json: a grid of (n, m) and the value its
tests/test_lxeb.py asserts), its closed form at n = 1 (2 / (m + 1)) and its
argument checks; the SVD dilation used by the non-uniform-loss sampler.

Tolerance: 1e-12 relative (the same closed form in double precision).
"""

import numpy as np
import pytest

from conftest import haar_unitary, load_golden
from piquasso_gb300.probabilities import lxe_ref_boson_sampling
from piquasso_gb300.sampling import expanded_interferometer


def test_lxe_ref_matches_reference_module():
    g = load_golden("lxeb_values.json")
    for c in g["boson_sampling"] + g["test_values"]:
        v = lxe_ref_boson_sampling(c["n"], c["m"])
        assert abs(v - c["value"]) <= 1e-12 * abs(c["value"]), c


@pytest.mark.parametrize("m", [1, 2, 7, 48])
def test_lxe_ref_single_photon(m):
    assert abs(lxe_ref_boson_sampling(1, m) - 2.0 / (m + 1)) < 1e-14


@pytest.mark.parametrize("n,m", [(10.0, 3), (-1, 3), (1, 0), (True, 3)])
def test_lxe_ref_invalid(n, m):
    with pytest.raises((TypeError, ValueError)):
        lxe_ref_boson_sampling(n, m)


def test_dilation_columns_of_the_input_modes():
    """Photons enter only the first d modes, so the first d columns of the
    dilation must be orthonormal (a loss-free embedding) and its upper-left
    block the lossy matrix itself."""
    U = haar_unitary(5, 3)
    M = U @ np.diag([0.9, 0.8, 0.7, 0.6, 0.5]) @ U.conj().T
    E = expanded_interferometer(M)
    assert np.allclose(E[:, :5].conj().T @ E[:, :5], np.eye(5), atol=1e-12)
    assert np.allclose(E[:5, :5], M, atol=1e-12)
