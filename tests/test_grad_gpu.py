"""GPU: ``permanent_grad`` (one batched Laplace walk per matrix row) against
the reference's gradient goldens (tests/golden/grad_cases.json) and the
double-double oracle, with batching, errors and edge cases.

Tolerance per entry: complex128 max(1e-10*|G_ij|, 1e-14*S_ij), complex64
max(1e-5*|G_ij|, 2^-22*S_ij), with S = grad_perm(|A|) the same gradient of the
entrywise absolute matrix (the scale of the sum's terms).
"""

import numpy as np
import pytest

import oracle
from conftest import as_matrix, haar_unitary, load_golden

pytestmark = pytest.mark.gpu


def _check(engine, A, rows, cols, want=None):
    A = np.asarray(A)
    got = engine.permanent_grad(A, rows, cols)
    assert got.shape == A.shape and got.dtype == A.dtype
    A128 = A.astype(np.complex128)
    dd = oracle.grad_perm(A128, rows, cols) if want is None else want
    scale = np.abs(oracle.grad_perm(np.abs(A128).astype(np.complex128), rows, cols))
    if A.dtype == np.complex64:
        tol = np.maximum(1e-5 * np.abs(dd), 2.0 ** -22 * scale)
    else:
        tol = np.maximum(1e-10 * np.abs(dd), 1e-14 * scale)
    err = np.abs(got.astype(np.complex128) - dd)
    assert np.all(err <= tol + 1e-300), (np.max(err - tol), rows, cols)
    return got


def test_reference_grad_goldens(engine):
    g = load_golden("grad_cases.json")
    for c in g["calls"] + g["random"]:
        A = as_matrix(c["matrix"]).astype(np.complex128)
        _check(engine, A, c["rows"], c["cols"], want=as_matrix(c["grad"]))
        _check(engine, A.astype(np.complex64), c["rows"], c["cols"])


def test_trivial_case_exact(engine):
    A = np.array([[1, 2, 3], [4, 5, 6], [7, 8, 9]], dtype=np.complex128)
    G = engine.permanent_grad(A, [1, 1, 1], [1, 1, 1])
    assert np.array_equal(G, np.array([[93, 78, 67], [42, 30, 22], [27, 18, 13]], dtype=np.complex128))


@pytest.mark.parametrize("n", [8, 12])
def test_haar_all_ones(engine, n):
    U = haar_unitary(2 * n, n)[:n, :n].copy()
    _check(engine, U, np.ones(n, int), np.ones(n, int))
    _check(engine, U.astype(np.complex64), np.ones(n, int), np.ones(n, int))


def test_repeated_rows_and_zero_columns(engine):
    U = haar_unitary(10, 3)[:7, :6].copy()
    rows = np.array([2, 0, 1, 3, 0, 1, 1])
    cols = np.array([3, 0, 2, 1, 0, 2])
    _check(engine, U, rows, cols)
    _check(engine, U.astype(np.complex64), rows, cols)


def test_batched_matches_single(engine):
    rng = np.random.default_rng(4)
    As = (rng.normal(size=(3, 2, 5, 5)) + 1j * rng.normal(size=(3, 2, 5, 5)))
    rows = rng.integers(0, 3, size=(3, 2, 5))
    cols = np.zeros_like(rows)
    for idx in np.ndindex(3, 2):  # cols: same total as rows, spread over the columns
        cols[idx] = np.bincount(rng.integers(0, 5, rows[idx].sum()), minlength=5)
    G = engine.permanent_grad(As, rows, cols)
    assert G.shape == As.shape
    for idx in np.ndindex(3, 2):
        # the batch and a single call may walk in different arithmetics (a
        # batch with a repeated column takes the FP64 Laplace walk for all
        # its matrices, an all-ones matrix alone the double-float one): they
        # agree to complex128 accuracy
        single = engine.permanent_grad(As[idx], rows[idx], cols[idx])
        scale = max(1.0, float(np.max(np.abs(single))))
        assert np.max(np.abs(G[idx] - single)) <= 1e-11 * scale
        _check(engine, As[idx], rows[idx], cols[idx])
    # shared multiplicities broadcast over the batch
    r1, c1 = np.array([1, 2, 0, 1, 1]), np.array([1, 1, 1, 1, 1])
    Gb = engine.permanent_grad(As, r1, c1)
    for idx in np.ndindex(3, 2):
        single = engine.permanent_grad(As[idx], r1, c1)
        assert np.max(np.abs(Gb[idx] - single)) <= 1e-11 * max(1.0, float(np.max(np.abs(single))))


def test_edge_cases(engine):
    A = np.array([[2.0 + 1j]], dtype=np.complex128)
    assert engine.permanent_grad(A, [1], [1])[0, 0] == 1.0
    assert engine.permanent_grad(A, [0], [0])[0, 0] == 0.0
    Z = np.zeros((3, 3), dtype=np.complex128)
    assert np.all(engine.permanent_grad(Z, [1, 1, 1], [1, 1, 1]) == 0)
    # no entry with rows_i > 0 and cols_j > 0: zeros, no sum check
    assert np.all(engine.permanent_grad(np.ones((2, 2), complex), [0, 0], [1, 0]) == 0)
    with pytest.raises(engine.PermanentInputError):
        engine.permanent_grad(np.ones((2, 2), complex), [1, 1], [1, 0])
    with pytest.raises(ValueError):
        engine.permanent_grad(np.ones((2, 2), complex), [1, -1], [0, 0])
