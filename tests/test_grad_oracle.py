"""CPU: the oracle's gradient restatement (oracle.grad_perm over the
double-double permanent) against the gradients that the reference's own
tests/jax_extensions/test_permanent_grad.py checks (tests/golden/grad_cases.json,
produced over the reference module's permanent and pinned by those tests'
golden assertions) and against seeded random cases.

Tolerance: 1e-12 * (1 + max |G|) per entry (both sides are complex128 sums
of the same minors; the golden side is the reference's own arithmetic).
"""

import numpy as np

import oracle
from conftest import as_matrix, load_golden


def _cases():
    g = load_golden("grad_cases.json")
    return g["calls"] + g["random"]


def test_golden_covers_reference_grad_tests():
    g = load_golden("grad_cases.json")
    assert len(g["tests_golden_checked"]) >= 10
    assert {"test_grad_perm_4_by_4", "test_grad_perm_6_by_6", "test_grad_perm_trivial_case"} <= set(
        g["tests_golden_checked"])


def test_oracle_grad_matches_golden():
    for c in _cases():
        A = as_matrix(c["matrix"]).astype(np.complex128)
        want = as_matrix(c["grad"])
        got = oracle.grad_perm(A, c["rows"], c["cols"])
        assert got.shape == want.shape
        assert np.max(np.abs(got - want)) <= 1e-12 * (1.0 + np.max(np.abs(want))), (c["rows"], c["cols"])


def test_oracle_grad_is_derivative():
    """Central finite differences of the dd permanent along each entry."""
    rng = np.random.default_rng(5)
    A = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    rows, cols = np.array([2, 0, 1, 1]), np.array([1, 1, 2, 0])
    G = oracle.grad_perm(A, rows, cols)
    h = 1e-6
    for i in range(4):
        for j in range(4):
            E = np.zeros_like(A)
            E[i, j] = h
            fd = (oracle.permanent(A + E, rows, cols) - oracle.permanent(A - E, rows, cols)) / (2 * h)
            assert abs(fd - G[i, j]) < 1e-6 * (1 + abs(G[i, j]))
