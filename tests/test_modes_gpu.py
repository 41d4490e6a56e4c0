"""GPU parity of the complex128 arithmetics (FP64 walk and double-float walk)
and of the run-based work split (short inner walks, many outer Gray steps per
lane, backward inner walks), against the double-double oracle.

Tolerance: complex128 max(1e-10*|perm|, 1e-14*perm(|A|)); the double-float
walk is additionally held to 1e-12 relative where |perm| is not tiny next to
perm(|A|) (it carries about 48 bits per operation).
"""

import numpy as np
import pytest

import oracle
from conftest import haar_unitary

pytestmark = pytest.mark.gpu


@pytest.fixture
def tuning(engine):
    old = engine.get_tuning()
    yield engine.set_tuning
    engine.set_tuning(old["items_per_smsp"], old["p_max"], old["seed_steps"])


def _tol(A, rows, cols, dd):
    return max(1e-10 * abs(dd), 1e-14 * oracle.perm_abs(A, rows, cols))


@pytest.mark.parametrize("mode", ["fp64", "df"])
@pytest.mark.parametrize("n", [10, 16, 20])
def test_modes_unit_multiplicities(engine, mode, n):
    U = haar_unitary(2 * n, 40 + n)[:n, :n].copy()
    o = np.ones(n, dtype=int)
    hi, lo = engine.permanent_dd(U, o, o, mode=mode)
    dd = oracle.permanent(U, o, o)
    assert abs(hi - dd) <= _tol(U, o, o, dd)
    if mode == "df":
        assert abs(hi - dd) <= 1e-12 * abs(dd) + 1e-14 * oracle.perm_abs(U, o, o) * 1e-3


@pytest.mark.parametrize("mode", ["fp64", "df"])
@pytest.mark.parametrize("seed", range(5))
def test_modes_repeated(engine, mode, seed):
    rng = np.random.default_rng(500 + seed)
    d = int(rng.integers(5, 14))
    n = int(rng.integers(6, 16))
    rows = np.bincount(rng.integers(0, d, n), minlength=d)
    cols = np.bincount(rng.integers(0, d, n), minlength=d)
    U = haar_unitary(d, seed) * (1.0 + 3.0 * rng.random((d, d)))  # not unitary: uneven scales
    hi, lo = engine.permanent_dd(U, rows, cols, mode=mode)
    dd = oracle.permanent(U, rows, cols)
    assert abs(hi - dd) <= _tol(U, rows, cols, dd), (hi, dd)


def test_df_large_dynamic_range(engine):
    # entries spanning many binades and a 6e30 permanent: column scaling keeps
    # the double-float sums in range
    A = np.full((3, 3), 1e10, dtype=complex)
    hi, _ = engine.permanent_dd(A, np.ones(3), np.ones(3), mode="df")
    assert abs(hi - 6e30) <= 1e-12 * 6e30
    rng = np.random.default_rng(9)
    B = (rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))) * np.exp(rng.uniform(-20, 20, size=(1, 8)))
    o = np.ones(8, dtype=int)
    hi, _ = engine.permanent_dd(B, o, o, mode="df")
    dd = oracle.permanent(B, o, o)
    assert abs(hi - dd) <= _tol(B, o, o, dd)


def test_df_falls_back_beyond_32_particles(engine):
    # 33 particles in few modes: the double-float domain ends, FP64 takes over
    rows = np.array([11, 11, 11])
    cols = np.array([11, 11, 11])
    U = haar_unitary(3, 2)
    hi, _ = engine.permanent_dd(U, rows, cols, mode="auto")
    dd = oracle.permanent(U, rows, cols)
    assert abs(hi - dd) <= _tol(U, rows, cols, dd)


@pytest.mark.parametrize("dtype,mode", [(np.complex128, "fp64"), (np.complex128, "df"), (np.complex64, "auto")])
def test_run_split_short_inner_walks(engine, tuning, dtype, mode):
    """p_max=4 forces inner walks of at most 4 codes at n=20, so every lane
    crosses several outer Gray steps and walks the inner codes backward half
    of the time (the default split would use long inner walks here)."""
    tuning(items_per_smsp=1, p_max=4, seed_steps=4096)
    n = 20
    U = haar_unitary(2 * n, 77)[:n, :n].copy()
    o = np.ones(n, dtype=int)
    rows = o.copy()
    rows[:4] = [2, 0, 2, 0]
    cols = np.ones(n, dtype=int)
    cols[5] = 2
    cols[6] = 0
    assert rows.sum() == cols.sum()
    for r, c in ((o, o), (rows, cols)):
        A = U.astype(dtype)
        dd = oracle.permanent(A.astype(np.complex128), r, c)
        if dtype == np.complex64:
            got = complex(engine.permanent(A, r, c))
            assert abs(got - dd) <= max(1e-5 * abs(dd), 2.0 ** -23 * oracle.perm_abs(A, r, c))
        else:
            got, _ = engine.permanent_dd(A, r, c, mode=mode)
            assert abs(got - dd) <= _tol(A, r, c, dd), (mode, got, dd)


def test_batch_mixed_column_counts(engine):
    """Problems with different numbers of distinct columns share one kernel
    through neutral padding columns."""
    rng = np.random.default_rng(21)
    d = 10
    U = haar_unitary(d, 21)
    R, C = [], []
    for b in range(30):
        n = int(rng.integers(1, 10))
        R.append(np.bincount(rng.integers(0, d, n), minlength=d))
        C.append(np.bincount(rng.integers(0, d, n), minlength=d))
    R, C = np.array(R), np.array(C)
    for mode in ("fp64", "df"):
        got = engine.permanent_batch(U, R, C, mode=mode)
        for b in range(len(R)):
            dd = oracle.permanent(U, R[b], C[b])
            assert abs(got[b] - dd) <= _tol(U, R[b], C[b], dd), (mode, b)


def test_auto_runs_the_fp64_walk_for_small_plans(engine):
    """Under "auto", a plain complex128 plan of at most 2^16 Gray-code steps runs
    the FP64 walk (exact to FP64 there, where the double-float walk rounds the
    scaled matrix to 2^-47); larger plans and an explicit "df" run the
    double-float walk."""
    from piquasso_gb300 import _lib

    for n, want in ((10, "plain_fp64_unit"), (17, "plain_fp64_unit"), (18, "plain_df_unit"), (22, "plain_df_unit")):
        U = haar_unitary(2 * n, 70 + n)[:n, :n].copy()
        o = np.ones(n, dtype=int)
        hi, _ = engine.permanent_dd(U, o, o, mode="auto")
        assert _lib.last_walk_kernel() == (want, n), (n, _lib.last_walk_kernel())
        dd = oracle.permanent(U, o, o)
        assert abs(hi - dd) <= _tol(U, o, o, dd)
    U = haar_unitary(20, 3)[:10, :10].copy()
    o = np.ones(10, dtype=int)
    engine.permanent_dd(U, o, o, mode="df")
    assert _lib.last_walk_kernel() == ("plain_df_unit", 10)
    assert abs(complex(engine.permanent(np.array([[4.2]]), [1], [1])) - 4.2) <= 4.2e-15
