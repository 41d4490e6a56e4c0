"""GPU: reusable plans executed as one CUDA graph (plain and Laplace forms),
on a scaled-down version of the batched-probabilities workload (uniform capped
compositions of the output photons)."""

import numpy as np
import pytest

import oracle
from conftest import haar_unitary
from piquasso_gb300 import workloads

pytestmark = pytest.mark.gpu


def _tol(A, rows, cols, dd):
    return max(1e-10 * abs(dd), 1e-14 * oracle.perm_abs(A, rows, cols))


@pytest.mark.parametrize("mode", ["auto", "fp64"])
def test_plan_batch_matches_oracle_and_repeats(engine, mode):
    d, n = 16, 8
    U = haar_unitary(d, 1)
    inp = np.array([1] * n + [0] * (d - n))
    pats = workloads.capped_compositions(n, d, 4, 48, seed=2)
    with engine.PermanentPlan(U, pats, inp, mode=mode) as plan:
        a = plan.run()
        b = plan.run()
        info = plan.info()
    assert np.array_equal(a, b)  # deterministic reductions
    assert info["steps"] == sum(workloads.gray_steps(p) for p in pats)
    for k in range(len(pats)):
        dd = oracle.permanent(U, pats[k], inp)
        assert abs(a[k] - dd) <= _tol(U, pats[k], inp, dd), k
    direct = engine.permanent_batch(U, pats, inp, mode=mode)
    assert np.allclose(direct, a, rtol=1e-12, atol=1e-15)


def test_plan_complex64_and_laplace(engine):
    d = 10
    U = haar_unitary(d, 3)
    rng = np.random.default_rng(8)
    R = np.zeros((12, d), dtype=int)
    C = np.zeros((12, d), dtype=int)
    for b in range(12):
        k = int(rng.integers(2, 8))
        C[b] = np.bincount(rng.choice(d, k, replace=False), minlength=d)
        R[b] = np.bincount(rng.integers(0, d, k - 1), minlength=d)
    with engine.PermanentPlan(U, R, C, form="laplace") as plan:
        lap = plan.run()
    direct = engine.permanent_laplace_batch(U, R, C)
    assert np.allclose(lap, direct, rtol=1e-12, atol=1e-15)
    U64 = U.astype(np.complex64)
    pats = np.stack([np.bincount(rng.integers(0, d, 5), minlength=d) for _ in range(10)])
    cols = np.array([1] * 5 + [0] * 5)
    with engine.PermanentPlan(U64, pats, cols) as plan:
        v = plan.run()
    assert v.dtype == np.complex64
    for k in range(len(pats)):
        dd = oracle.permanent(U64.astype(np.complex128), pats[k], cols)
        assert abs(v[k] - dd) <= max(1e-5 * abs(dd), 2.0 ** -23 * oracle.perm_abs(U64, pats[k], cols))


@pytest.mark.parametrize("dtype,mode", [(np.complex64, "auto"), (np.complex128, "auto"), (np.complex128, "fp64")])
@pytest.mark.parametrize("seed", range(3))
def test_random_batches_against_oracle(engine, dtype, mode, seed):
    """Randomised batches that exercise the planner's work split: problems of
    very different sizes (longest items first, outputs in caller order), whole
    warps and groups of items with empty trailing items, 1..20 distinct
    columns padded to the batch's widest (shared-memory tables from 17
    columns), repeated rows and columns, and constant (empty) problems."""
    rng = np.random.default_rng(1000 + seed)
    d = 22
    U = haar_unitary(d, 50 + seed).astype(dtype)
    R, C = [], []
    for b in range(40):
        n = int(rng.integers(0, 19)) if b % 13 else 0
        rows = np.bincount(rng.integers(0, d, n), minlength=d)
        if b % 3 == 0:  # distinct input columns
            cols = np.zeros(d, dtype=int)
            cols[rng.permutation(d)[:n]] = 1
        else:
            cols = np.bincount(rng.integers(0, d, n), minlength=d)
        R.append(rows)
        C.append(cols)
    R, C = np.stack(R), np.stack(C)
    if mode == "auto":
        got = engine.permanent_batch(U, R, C)
    else:
        with engine.PermanentPlan(U, R, C, mode=mode) as p:
            got = p.run()
    for b in range(len(R)):
        dd = oracle.permanent(U.astype(np.complex128), R[b], C[b])
        if dtype == np.complex64:
            tol = max(1e-5 * abs(dd), 2.0 ** -22 * oracle.perm_abs(U.astype(np.complex128), R[b], C[b]))
        else:
            tol = max(1e-10 * abs(dd), 1e-14 * oracle.perm_abs(U.astype(np.complex128), R[b], C[b]))
        assert abs(complex(got[b]) - dd) <= tol, (b, got[b], dd)
