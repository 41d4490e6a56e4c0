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


def _oracle_batch(U, rows, cols, mode="auto"):
    """permanent_batch restated on the double-double oracle (CPU)."""
    import oracle

    R = np.atleast_2d(np.asarray(rows))
    C = np.asarray(cols)
    if C.ndim == 1:
        C = np.broadcast_to(C, (R.shape[0], C.shape[0]))
    return np.array([oracle.permanent(np.asarray(U, dtype=np.complex128), r, c) for r, c in zip(R, C)])


def test_detection_probabilities_host_logic(monkeypatch):
    """detection_probabilities with the engine's batch call replaced by the
    oracle: a superposition of two inputs of the same photon number, and
    patterns of another photon number (probability 0); against the formula
    |sum_k c_k perm(U; y, x_k) / sqrt(prod y! prod x_k!)|^2 evaluated directly."""
    from math import factorial

    from piquasso_gb300 import probabilities

    monkeypatch.setattr(probabilities, "permanent_batch", _oracle_batch)
    import oracle

    d = 5
    rng = np.random.default_rng(2)
    Z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    U, _ = np.linalg.qr(Z)
    X = np.array([[1, 1, 1, 0, 0], [2, 0, 0, 1, 0]])
    c = np.array([0.6, 0.8j])
    Y = np.array([[1, 0, 1, 1, 0], [0, 0, 3, 0, 0], [0, 2, 0, 0, 1], [1, 1, 0, 0, 0]])
    got = probabilities.detection_probabilities(U, Y, X, c)
    for y, g in zip(Y, got):
        if y.sum() != 3:
            assert g == 0.0
            continue
        amp = 0j
        for ck, x in zip(c, X):
            norm = np.sqrt(np.prod([factorial(v) for v in y]) * np.prod([factorial(v) for v in x]))
            amp += ck * oracle.permanent(U, y, x) / norm
        assert abs(g - abs(amp) ** 2) <= 1e-13 * max(1.0, abs(amp) ** 2)


def test_metropolis_log_target_host_logic(monkeypatch):
    """log p(y) = 2 log|perm(U[y, in])| - sum log y! on the oracle's permanents."""
    from math import lgamma

    from piquasso_gb300 import metropolis

    monkeypatch.setattr(metropolis, "permanent_batch", _oracle_batch)
    import oracle

    d = 6
    rng = np.random.default_rng(7)
    Z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    U, _ = np.linalg.qr(Z)
    inp = np.array([1, 1, 1, 1, 0, 0])
    Y = np.array([[1, 1, 1, 1, 0, 0], [4, 0, 0, 0, 0, 0], [0, 2, 0, 1, 0, 1]])
    lp = metropolis.log_target(U.astype(np.complex64), Y, inp)
    for y, v in zip(Y, lp):
        p = abs(oracle.permanent(U.astype(np.complex64).astype(np.complex128), y, inp)) ** 2
        want = np.log(p) - sum(lgamma(k + 1.0) for k in y)
        assert abs(v - want) <= 1e-9 * max(1.0, abs(want))
