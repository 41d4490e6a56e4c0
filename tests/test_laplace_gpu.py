"""GPU parity of ``permanent_laplace`` against the reference's outputs and the
double-double oracle, and the reference's seeded sampler golden driven by it.

Tolerance: complex128 max(1e-10*|L_l|, 1e-14*perm(|A|) with column l lowered);
complex64 max(1e-5*|L_l|, 2^-23*perm(|A|)).
"""

import numpy as np
import pytest

import oracle
from conftest import as_complex, as_matrix, haar_unitary, load_golden
from oracle import sampler as osampler

pytestmark = pytest.mark.gpu


def _abs_scales(A, rows, cols):
    A = np.abs(np.asarray(A, dtype=np.complex128)).astype(np.complex128)
    out = []
    for l in range(len(cols)):
        c = np.array(cols).copy()
        c[l] = max(c[l] - 1, 0)
        out.append(abs(oracle.permanent_laplace_dd(A, rows, np.array(cols))[l]))
    return np.array(out)


def _check(engine, A, rows, cols, ref=None):
    A = np.asarray(A)
    got = engine.permanent_laplace(A, rows, cols)
    dd = oracle.permanent_laplace_dd(np.asarray(A, dtype=np.complex128), rows, cols)
    assert got.shape == dd.shape
    scales = _abs_scales(A, rows, cols)
    if A.dtype == np.complex64:
        assert got.dtype == np.complex64
        t = np.maximum(1e-5 * np.abs(dd), 2.0 ** -23 * scales)
    else:
        assert got.dtype == np.complex128
        t = np.maximum(1e-10 * np.abs(dd), 1e-14 * scales)
        if ref is not None:
            assert np.all(np.abs(got - ref) <= t + 1e-300)
    assert np.all(np.abs(got - dd) <= t + 1e-300), (got, dd, t)
    return got


def test_reference_random_laplace(engine):
    data = load_golden("random_cases.json")
    for case in data["laplace"]:
        A = as_matrix(case["matrix"])
        ref = np.array([as_complex(z) for z in case["result"]])
        got = _check(engine, A, case["rows"], case["cols"], ref if A.dtype == np.complex128 else None)
        assert str(got.dtype) == case["result_dtype"]


@pytest.mark.parametrize("k", [2, 5, 9, 14, 18])
def test_sampler_shaped_laplace(engine, k):
    # step k of the sampler: (k-1) output photons over k input columns
    rng = np.random.default_rng(k)
    d = 2 * k + 2
    U = haar_unitary(d, k)
    cols = np.ones(k, dtype=int)
    sample = np.bincount(rng.integers(0, d, k - 1), minlength=d)
    A = U[:, :k][sample > 0].copy()
    rows = sample[sample > 0]
    _check(engine, A, rows, cols)
    _check(engine, A.astype(np.complex64), rows, cols)


def test_laplace_edge_cases(engine):
    assert np.array_equal(engine.permanent_laplace(np.eye(2), [0, 0], [1, 1]), np.array([1.0 + 0j]))
    assert engine.permanent_laplace(np.eye(2, dtype=np.complex64), [1, 0], [1, 1]).dtype == np.complex64
    # a zero-multiplicity column keeps exponent 0 (reference semantics)
    A = haar_unitary(4, 1)[:3].copy()
    _check(engine, A, [1, 1, 0], [1, 2, 0, 0])
    # repeated columns
    _check(engine, A, [2, 1, 1], [2, 1, 2, 0])


def test_seeded_sampler_golden(engine):
    g = load_golden("sampler_seeded.json")
    U = as_matrix(g["U"])
    samples = osampler.generate_samples(np.array(g["input"]), g["shots"], engine.permanent_laplace, U, g["seed"])
    assert [list(s) for s in samples] == g["generated_samples"]
    assert [list(s) for s in osampler.result_samples(samples, g["seed"])] == g["expected_samples"]


def test_double_float_laplace_matches_fp64_at_full_size(engine):
    """complex128 Laplace permanents take the double-float walk by default
    (all-ones columns); at the sampler's full size (23 output photons with
    collisions, 24 unit input columns, d=48) they agree with the FP64 walk
    within the complex128 bound max(1e-10 |value|, 1e-14 perm(|A|)) -- the
    permanent of |A| with column l lowered bounds every output l."""
    rng = np.random.default_rng(12)
    d, n = 48, 24
    U = haar_unitary(d, 3)
    cols = np.array([1] * n + [0] * (d - n))
    R = np.stack([np.bincount(rng.integers(0, d, n - 1), minlength=d) for _ in range(64)])
    with engine.PermanentPlan(U, R, cols, form="laplace", mode="df") as p:
        df = p.run()
    with engine.PermanentPlan(U, R, cols, form="laplace", mode="fp64") as p:
        f64 = p.run()
    with engine.PermanentPlan(np.abs(U).astype(np.complex128), R, cols, form="laplace", mode="fp64") as p:
        pabs = np.abs(p.run())
    assert df.shape == f64.shape == (64, d)
    bound = np.maximum(1e-10 * np.abs(f64), 1e-14 * pabs)
    assert np.all(np.abs(df - f64) <= bound), float(np.max(np.abs(df - f64) / np.maximum(bound, 1e-300)))
    # the default entry point (double-float) agrees as well
    direct = engine.permanent_laplace_batch(U, R, np.broadcast_to(cols, R.shape))
    assert np.all(np.abs(direct - f64) <= bound)


def test_double_float_laplace_repeated_columns(engine):
    """Repeated input columns (multi-photon input modes) take the general
    double-float Laplace kernel: each output keeps cols_l - 1 factors of its
    column.  Against the FP64 walk within the complex128 bound."""
    rng = np.random.default_rng(31)
    d, n = 30, 19
    U = haar_unitary(d, 7)
    C = []
    for b in range(48):
        c = np.zeros(d, dtype=int)
        c[rng.permutation(d)[:n - 4]] = 1
        c[rng.permutation(np.nonzero(c)[0])[:4]] += 1  # four doubly occupied input modes
        C.append(c)
    C = np.stack(C)
    R = np.stack([np.bincount(rng.integers(0, d, n - 1), minlength=d) for _ in range(48)])
    with engine.PermanentPlan(U, R, C, form="laplace", mode="df") as p:
        df = p.run()
    with engine.PermanentPlan(U, R, C, form="laplace", mode="fp64") as p:
        f64 = p.run()
    for b in range(len(R)):
        for l in np.nonzero(C[b])[0]:
            cl = C[b].copy()
            cl[l] -= 1
            bound = max(1e-10 * abs(f64[b, l]), 1e-14 * oracle.perm_abs(U, R[b], cl))
            assert abs(df[b, l] - f64[b, l]) <= bound, (b, l)
    dd = oracle.permanent_laplace_dd(U, R[0], C[0])
    nz = C[0] > 0
    assert np.allclose(df[0][nz], dd[nz], rtol=1e-10, atol=0)
