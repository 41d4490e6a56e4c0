"""GPU parity of ``permanent`` / ``permanent_batch`` against the reference's
golden vectors and the double-double oracle.

Tolerances (written here, used throughout):
  complex128: |gpu - ref| <= max(1e-10*|perm|, 1e-14*perm(|A|))
  complex64:  |gpu - dd(A64)| <= max(1e-5*|perm|, 1e-6*S64) where S64 is the
              rounding scale of FP32 terms: 2^-23 * perm(|A|) (the same
              bound with the complex64 unit roundoff in place of 1e-14)
"""

import numpy as np
import pytest

import oracle
from conftest import as_complex, as_matrix, haar_unitary, load_golden

pytestmark = pytest.mark.gpu


def tol128(A, rows, cols, value):
    return max(1e-10 * abs(value), 1e-14 * oracle.perm_abs(np.asarray(A, dtype=np.complex128), rows, cols))


def tol64(A, rows, cols, value):
    pa = oracle.perm_abs(np.asarray(A, dtype=np.complex128), rows, cols)
    return max(1e-5 * abs(value), 2.0 ** -23 * pa)


def _check(engine, A, rows, cols, ref_value=None):
    A = np.asarray(A)
    got = engine.permanent(A, rows=rows, cols=cols)
    dd = oracle.permanent(np.asarray(A, dtype=np.complex128), rows, cols)
    if A.dtype == np.complex64:
        assert got.dtype == np.complex64
        assert abs(complex(got) - dd) <= tol64(A, rows, cols, dd), (got, dd)
    else:
        assert got.dtype == np.complex128
        t = tol128(A, rows, cols, dd)
        assert abs(complex(got) - dd) <= t, (got, dd, t)
        if ref_value is not None:
            assert abs(complex(got) - ref_value) <= t, (got, ref_value, t)
    return got


@pytest.mark.parametrize("fixture", ["permanent_known_answers.json", "jax_unit_cases.json"])
def test_reference_known_answers(engine, fixture):
    data = load_golden(fixture)
    assert data["calls"], "fixture holds no cases"
    for case in data["calls"]:
        A = as_matrix(case["matrix"])
        got = engine.permanent(A, rows=case["rows"], cols=case["cols"])
        assert str(got.dtype) == case["result_dtype"]
        ref = as_complex(case["result"])
        A128 = np.asarray(A, dtype=np.complex128)
        t = max(1e-10 * abs(ref), 1e-14 * oracle.perm_abs(A128, case["rows"], case["cols"]))
        if got.dtype == np.complex64:
            t = max(1e-5 * abs(ref), 2.0 ** -23 * oracle.perm_abs(A128, case["rows"], case["cols"]), 1e-6)
        assert abs(complex(got) - ref) <= t, (case["rows"], case["cols"], got, ref)


def test_reference_random_cases(engine):
    data = load_golden("random_cases.json")
    for case in data["permanent"]:
        A = as_matrix(case["matrix"])
        got = engine.permanent(A, rows=case["rows"], cols=case["cols"])
        assert str(got.dtype) == case["result_dtype"]
        dd = as_complex(case["dd"])
        if got.dtype == np.complex64:
            t = max(1e-5 * abs(dd), 2.0 ** -23 * case["perm_abs"])
        else:
            t = max(1e-10 * abs(dd), 1e-14 * case["perm_abs"])
            assert abs(complex(got) - as_complex(case["result"])) <= t
        assert abs(complex(got) - dd) <= t, (case["rows"], case["cols"], got, dd)


def test_config14_cases(engine):
    data = load_golden("config_14.json")
    for case in data["cases"]:
        A = as_matrix(case["matrix"])
        got = engine.permanent(A, rows=case["rows"], cols=case["cols"])
        dd = as_complex(case["dd_hi"]) + as_complex(case["dd_lo"])
        if A.dtype == np.complex64:
            t = max(1e-5 * abs(dd), 2.0 ** -23 * case["perm_abs"])
        else:
            t = max(1e-10 * abs(dd), 1e-14 * case["perm_abs"])
            assert abs(complex(got) - as_complex(case["result"])) <= t
        assert abs(complex(got) - dd) <= t, (case["label"], got, dd)


@pytest.mark.parametrize("n", [16, 18, 20])
def test_haar_unit_multiplicities(engine, n):
    U = haar_unitary(2 * n, n)[:n, :n].copy()
    ones = np.ones(n, dtype=int)
    got = _check(engine, U, ones, ones)
    hi, lo = engine.permanent_dd(U, ones, ones)
    assert hi == complex(got)
    _check(engine, U.astype(np.complex64), ones, ones)


@pytest.mark.parametrize("seed", range(6))
def test_repeated_rows_and_columns(engine, seed):
    rng = np.random.default_rng(100 + seed)
    d = int(rng.integers(6, 16))
    n = int(rng.integers(8, 18))
    rows = np.bincount(rng.integers(0, d, n), minlength=d)
    cols = np.bincount(rng.integers(0, d, n), minlength=d)
    U = haar_unitary(d, seed)
    _check(engine, U, rows, cols)
    _check(engine, U.astype(np.complex64), rows, cols)


def test_edge_cases(engine):
    # empty, all-zero multiplicities, 1x1, zero entry, identity, large values
    assert complex(engine.permanent(np.zeros((0, 0)), [], [])) == 1.0
    assert complex(engine.permanent(np.eye(3), [0, 0, 0], [0, 0, 0])) == 1.0
    assert abs(complex(engine.permanent(np.array([[4.2]]), [1], [1])) - 4.2) < 1e-14
    assert complex(engine.permanent(np.array([[0j]]), [1], [1])) == 0.0
    assert abs(complex(engine.permanent(np.eye(8, dtype=complex), np.ones(8), np.ones(8))) - 1.0) < 1e-14
    big = engine.permanent(np.full((3, 3), 1e10, dtype=complex), np.ones(3), np.ones(3))
    assert abs(complex(big) - 6e30) <= 1e-10 * 6e30
    # one row with all photons: perm = N! prod a_j^{c_j} / prod ... as the reference computes
    A = np.array([[0.3 + 0.1j, -0.2 + 0.4j, 0.5 - 0.3j]])
    _check(engine, A, [4], [1, 2, 1])
    # a single photon
    _check(engine, A, [1], [0, 1, 0])


def test_errors(engine):
    with pytest.raises(RuntimeError):
        engine.permanent(np.eye(2), [1, 1], [2, 1])
    with pytest.raises(ValueError):
        engine.permanent(np.eye(2), [1, 1], [2, 1])
    with pytest.raises(ValueError):
        engine.permanent(np.eye(2), [1, 1, 0], [1, 1])
    with pytest.raises(TypeError):
        engine.permanent(np.eye(2, dtype=np.clongdouble), [1, 1], [1, 1])
    with pytest.raises(engine.PermanentTooLarge):
        engine.permanent(np.ones((2, 40)), [20, 20], np.ones(40))


def test_dtype_rules(engine):
    o = np.ones(2, dtype=int)
    m = np.array([[1, 2], [3, 4]])
    for dt, want in ((np.float32, np.complex64), (np.float64, np.complex128), (np.int16, np.complex64),
                     (np.int32, np.complex128), (np.int64, np.complex128), (np.complex64, np.complex64),
                     (np.complex128, np.complex128), (np.uint8, np.complex64)):
        r = engine.permanent(m.astype(dt), o, o)
        assert r.dtype == want and r.shape == () and abs(complex(r) - 10) < 1e-5
    assert engine.permanent([[1, 2], [3, 4]], [1, 1], [1, 1]).dtype == np.complex64
    # forcecast multiplicities
    assert abs(complex(engine.permanent(np.eye(2), np.array([1.7, 1.2]), [1, 1])) - 1.0) < 1e-14


def test_batch_matches_single_calls(engine):
    rng = np.random.default_rng(5)
    d, n = 12, 9
    U = haar_unitary(d, 3)
    cols = np.bincount(rng.integers(0, d, n), minlength=d)
    R = np.stack([np.bincount(rng.integers(0, d, n), minlength=d) for _ in range(40)])
    R[3] = 0
    R[3, 0] = n  # all photons in one mode
    got = engine.permanent_batch(U, R, cols)
    for b in range(R.shape[0]):
        dd = oracle.permanent(U, R[b], cols)
        assert abs(got[b] - dd) <= tol128(U, R[b], cols, dd), b
    got64 = engine.permanent_batch(U.astype(np.complex64), R, cols)
    for b in range(R.shape[0]):
        dd = oracle.permanent(U.astype(np.complex64).astype(np.complex128), R[b], cols)
        assert abs(got64[b] - dd) <= tol64(U.astype(np.complex64), R[b], cols, dd), b


def test_large_n_properties(engine):
    """Size-independent identities at n=26: transpose, conjugation, row scaling."""
    n = 26
    U = haar_unitary(2 * n, 26)[:n, :n].copy()
    ones = np.ones(n, dtype=int)
    p = complex(engine.permanent(U, ones, ones))
    pt = complex(engine.permanent(U.T.copy(), ones, ones))
    pc = complex(engine.permanent(U.conj(), ones, ones))
    V = U.copy()
    V[3] *= 2.0  # exact scaling by a power of two
    ps = complex(engine.permanent(V, ones, ones))
    scale = np.sum(np.abs(U), axis=0).prod()  # >= perm(|A|): a safe error scale
    t = max(1e-10 * abs(p), 1e-14 * scale)
    assert abs(pt - p) <= 2 * t
    assert abs(pc - p.conjugate()) <= 2 * t
    assert abs(ps - 2 * p) <= 4 * t


def test_cpu_baseline_port_agrees_with_engine(engine):
    """The CPU baseline (the reference's method restated, oracle/perm_port.cpp)
    computes the same permanents as the engine on this host, whatever its
    architecture (the reference keeps the term's sign in a plain char, which
    is unsigned on aarch64)."""
    oracle.build.build(with_reference=False)
    for n in (8, 14):
        A = haar_unitary(2 * n, 1)[:n, :n].copy()
        o = np.ones(n, dtype=int)
        r2, c2 = o.copy(), o.copy()
        r2[0] -= 1
        c2[1] -= 1
        for r, c in ((o, o), (r2, c2)):
            want = engine.permanent(A, r, c)
            got = oracle.port_permanent(A, r, c)
            assert abs(got - want) <= 1e-10 * abs(want)
        lap = oracle.port_laplace(A, r2, o)
        assert np.allclose(lap, engine.permanent_laplace(A, r2, o), rtol=1e-10, atol=0)


def test_complex64_shared_table_batches_match_oracle(engine):
    """17..24 distinct columns: the complex64 walk stages each problem's
    prefix table in shared memory, restaged when a block moves on to another
    problem of the batch; unit columns (all-ones kernel) and one doubled input
    column (repeated-column kernel), rows with collisions."""
    rng = np.random.default_rng(41)
    d = 34
    U = haar_unitary(d, 41).astype(np.complex64)
    for cols in (np.array([1] * 17 + [0] * 17), np.array([1] * 17 + [2] + [0] * 16)):
        n = int(cols.sum())
        R = np.stack([np.bincount(rng.integers(0, d, n), minlength=d) for _ in range(24)])
        got = engine.permanent_batch(U, R, cols)
        for b in range(len(R)):
            dd = oracle.permanent(U.astype(np.complex128), R[b], cols)
            assert abs(got[b] - dd) <= tol64(U, R[b], cols, dd), b


def test_complex64_target_batch_matches_complex128(engine):
    """The Metropolis target shape at full size (n=24 photons in 48 modes, 512
    patterns with occupations <= 4, one batched launch): complex64 against
    the double-float complex128 path (relative error ~1e-12), within the
    complex64 bound max(1e-5 |perm|, 2^-22 perm(|A|))."""
    rng = np.random.default_rng(7)
    d, n = 48, 24
    U = haar_unitary(d, 3)
    inp = np.array([1] * n + [0] * (d - n))
    R = []
    while len(R) < 512:
        r = np.bincount(rng.integers(0, d, n), minlength=d)
        if r.max() <= 4:
            R.append(r)
    R = np.stack(R)
    got = engine.permanent_batch(U.astype(np.complex64), R, inp).astype(np.complex128)
    ref = engine.permanent_batch(U, R, inp)
    pabs = engine.permanent_batch(np.abs(U).astype(np.complex128), R, inp).real
    err = np.abs(got - ref)
    bound = np.maximum(1e-5 * np.abs(ref), 2.0 ** -22 * pabs)
    assert np.all(err <= bound), (np.max(err / bound), int(np.argmax(err / bound)))
