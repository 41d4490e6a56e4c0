"""GPU parity at the sizes the throughput numbers are quoted on, and of every
separately compiled walk kernel.

* Every (walk table, column count) instantiation — plain and Laplace, FP64,
  double-float and complex64, unit and repeated columns, 1..32 columns —
  against the double-double oracle.  pqg_last_walk_kernel reports which
  instantiation a call launched, so each case asserts that the intended
  kernel ran.  The output photons sit in few modes (at most 8 each), so the
  Gray-code space stays small (<= 9^3 * 8 codes) and the oracle cheap.
* Single large permanents (leading n x n block of Haar(2n), seed 0, unit
  multiplicities, the inputs of the single-permanent benchmark): n = 24 and
  26 against the double-double oracle, n = 28 against the oracle and the
  reference's CPU method, n = 30 against the reference's CPU method, in the
  FP64, double-float and complex64 arithmetics.
* 64 patterns of the batched-probability workload (d = 40, n = 20, 4096
  uniform capped compositions) and 64 proposals of the Metropolis target
  batch (d = 48, n = 24, complex64), each against the oracle.

Tolerances (the reference method's contract, reference src/permanent.cpp:49-264):
  complex128: |gpu - dd| <= max(1e-10*|perm|, 1e-14*perm(|A|))
  complex64:  |gpu - dd(A64)| <= max(1e-5*|perm|, 2^-23*perm(|A|)) for the
              Haar inputs; for the instantiation sweep, whose inputs put up
              to 8 photons in a mode and cancel strongly (sum |terms| ~ 450
              |perm|), the first-order forward error bound of FP32 products of
              N = sum(cols) factors, max(1e-5*|perm|, (N+2)*2^-24*perm(|A|)).
              (There a FP32 emulation of the kernel's exact operation order
              reproduces its result to the last bit; 2^-23 perm(|A|), two unit
              roundoffs, is below what N-factor FP32 products guarantee, and
              the reference's own complex64 method exceeds 1e-5*|perm| on the
              same inputs.)
"""

import numpy as np
import pytest

import oracle
from conftest import haar_unitary

pytestmark = pytest.mark.gpu

TOL128 = (1e-10, 1e-14)
TOL64 = (1e-5, 2.0 ** -23)


def _rows_in_few_modes(N, per=8):
    """N photons over ceil(N/per) modes, as evenly as possible."""
    k = max(1, -(-N // per))
    r = np.full(k, N // k, dtype=np.int64)
    r[: N % k] += 1
    return r


def _case(form, nc, unit, seed):
    """(matrix, rows, cols) with exactly nc distinct nonzero columns.

    Plain form: N = sum(cols) photons.  Laplace form: sum(rows) =
    sum(cols) - 1; the repeated-column Laplace case also carries one
    zero-multiplicity column (the shared extra output)."""
    cols = np.ones(nc, dtype=np.int64)
    if not unit:
        cols[0] = 2
    if form == "laplace" and not unit:
        cols = np.append(cols, 0)
    N = int(cols.sum()) - (1 if form == "laplace" else 0)
    rows = _rows_in_few_modes(N)
    U = haar_unitary(len(cols) + len(rows), seed)[: len(rows), : len(cols)].copy()
    return U, rows, cols


def _expected_table(form, arith, unit, nc):
    if form == "plain":
        base = {"fp64": "plain_fp64", "df": "plain_df", "c64": "plain_c64"}[arith]
        return base + ("_unit" if unit else "")
    if arith == "fp64":
        return "laplace_fp64"
    if arith == "df":
        return "laplace_df_unit" if unit and nc <= 25 else "laplace_df"
    # unit columns up to 24: the two-code walk over code-pair tables; wider: the general walk
    return "laplace_c64_unit" if unit and nc <= 24 else "laplace_c64"


def _column_counts(form, arith, unit):
    lo = 2 if (form == "laplace" and unit) else 1  # one unit column and no row photon: no walk
    hi = 32
    if form == "plain" and arith == "df" and not unit:
        hi = 31  # 33 photons leave the double-float domain (the FP64 walk takes over)
    return range(lo, hi + 1)


def _run(engine, monkeypatch, form, arith, A, rows, cols):
    if arith == "c64":
        A = A.astype(np.complex64)
    if form == "plain":
        if arith == "c64":
            got = complex(engine.permanent(A, rows, cols))
        else:
            got = engine.permanent_dd(A, rows, cols, mode=arith)[0]
        return A, np.array([got])
    if arith == "fp64":
        monkeypatch.setenv("PQG_C128_MODE", "fp64")
    else:
        monkeypatch.delenv("PQG_C128_MODE", raising=False)
    got = engine.permanent_laplace(A, rows, cols).astype(np.complex128)
    monkeypatch.delenv("PQG_C128_MODE", raising=False)
    return A, got


def _oracle(form, A, rows, cols):
    A128 = np.asarray(A, dtype=np.complex128)
    if form == "plain":
        return (np.array([oracle.permanent(A128, rows, cols)]),
                np.array([oracle.perm_abs(A128, rows, cols)]))
    want = oracle.permanent_laplace_dd(A128, rows, cols)
    scale = np.abs(oracle.permanent_laplace_dd(np.abs(A128).astype(np.complex128), rows, cols).real)
    return want, scale


@pytest.mark.parametrize("form,arith,unit", [
    ("plain", "fp64", True), ("plain", "fp64", False),
    ("plain", "df", True), ("plain", "df", False),
    ("plain", "c64", True), ("plain", "c64", False),
    ("laplace", "fp64", True), ("laplace", "fp64", False),
    ("laplace", "df", True), ("laplace", "df", False),
    ("laplace", "c64", True), ("laplace", "c64", False),
])
def test_every_walk_instantiation_matches_oracle(engine, monkeypatch, form, arith, unit):
    from piquasso_gb300 import _lib

    cases = [(nc, False) for nc in _column_counts(form, arith, unit)]
    if form == "laplace" and unit:
        # unit columns beside a zero-multiplicity column (the exact sampler's
        # steps): the walk's extra output shared by the zero columns
        cases += [(nc, True) for nc in _column_counts(form, arith, unit)]
    for nc, zero_col in cases:
        A, rows, cols = _case(form, nc, unit, seed=1000 + nc)
        if zero_col:
            cols = np.append(cols, 0)
            A = haar_unitary(len(cols) + len(rows), 2000 + nc)[: len(rows), : len(cols)].copy()
        n_factors = int(cols.sum())
        rel, absf = (1e-5, (n_factors + 2) * 2.0 ** -24) if arith == "c64" else TOL128
        A, got = _run(engine, monkeypatch, form, arith, A, rows, cols)
        table, ran_nc = _lib.last_walk_kernel()
        assert (table, ran_nc) == (_expected_table(form, arith, unit, nc), nc), (form, arith, unit, nc, zero_col)
        want, scale = _oracle(form, A, rows, cols)
        assert got.shape == want.shape, (nc, got.shape, want.shape)
        tol = np.maximum(rel * np.abs(want), absf * scale)
        err = np.abs(got - want)
        assert np.all(err <= tol), (form, arith, unit, nc, zero_col, float(np.max(err / tol)))


def _leading_block(n):
    return haar_unitary(2 * n, 0)[:n, :n].copy()


def _check_full(engine, n, arith, want, pabs):
    U = _leading_block(n)
    o = np.ones(n, dtype=int)
    from piquasso_gb300 import _lib

    if arith == "c64":
        U64 = U.astype(np.complex64)
        got = complex(engine.permanent(U64, o, o))
        rel, absf = TOL64
    else:
        got = engine.permanent_dd(U, o, o, mode=arith)[0]
        rel, absf = TOL128
    table, ran_nc = _lib.last_walk_kernel()
    assert ran_nc == n and table == {"fp64": "plain_fp64_unit", "df": "plain_df_unit", "c64": "plain_c64_unit"}[arith]
    tol = max(rel * abs(want), absf * pabs)
    assert abs(got - want) <= tol, (n, arith, got, want, abs(got - want) / tol)
    return got


@pytest.mark.parametrize("n", [24, 26])
def test_single_large_permanent_against_dd_oracle(engine, n):
    U = _leading_block(n)
    o = np.ones(n, dtype=int)
    want = oracle.permanent(U, o, o)
    pabs = oracle.perm_abs(U, o, o)
    df = _check_full(engine, n, "df", want, pabs)
    fp = _check_full(engine, n, "fp64", want, pabs)
    # both complex128 arithmetics carry ~48 bits or more per operation: far
    # inside the contract at these sizes
    assert abs(df - want) <= 1e-11 * abs(want) + 1e-16 * pabs
    assert abs(fp - want) <= 1e-11 * abs(want) + 1e-16 * pabs
    want64 = oracle.permanent(U.astype(np.complex64).astype(np.complex128), o, o)
    _check_full(engine, n, "c64", want64, pabs)


def test_n28_against_dd_oracle_and_reference_method(engine):
    n = 28
    U = _leading_block(n)
    o = np.ones(n, dtype=int)
    ref = complex(oracle.port_permanent(U, o, o))  # the reference's CPU method
    pabs = float(abs(oracle.port_permanent(np.abs(U).astype(np.complex128), o, o)))  # no cancellation
    want = oracle.permanent(U, o, o)
    for arith in ("df", "fp64"):
        got = _check_full(engine, n, arith, want, pabs)
        assert abs(got - ref) <= max(1e-10 * abs(ref), 1e-14 * pabs), (arith, got, ref)
    want64 = oracle.permanent(U.astype(np.complex64).astype(np.complex128), o, o)
    _check_full(engine, n, "c64", want64, pabs)


def test_n30_against_reference_method(engine):
    n = 30
    U = _leading_block(n)
    o = np.ones(n, dtype=int)
    ref = complex(oracle.port_permanent(U, o, o))
    pabs = float(abs(oracle.port_permanent(np.abs(U).astype(np.complex128), o, o)))
    for arith in ("df", "fp64"):
        _check_full(engine, n, arith, ref, pabs)
    # complex64 against the reference method run on the complex64-rounded
    # matrix in complex128 arithmetic
    ref64 = complex(oracle.port_permanent(U.astype(np.complex64).astype(np.complex128), o, o))
    _check_full(engine, n, "c64", ref64, pabs)


def test_batched_probability_workload_against_oracle(engine):
    """The benchmarked batch (4096 uniform capped compositions of 20 photons
    into 40 modes, Haar(40) seed 1, inputs in modes 0..19), run as one plan;
    64 of its patterns checked against the oracle."""
    from piquasso_gb300 import workloads

    d, n = 40, 20
    U = workloads.haar_unitary(d, 1)
    patterns = workloads.capped_compositions(n, d, 4, 4096, seed=1)
    inp = np.array([1] * n + [0] * (d - n))
    plan = engine.PermanentPlan(U, patterns, inp)
    try:
        plan.run()
        got = plan.read()
    finally:
        plan.close()
    for b in np.linspace(0, len(patterns) - 1, 64).astype(int):
        want = oracle.permanent(U, patterns[b], inp)
        tol = max(1e-10 * abs(want), 1e-14 * oracle.perm_abs(U, patterns[b], inp))
        assert abs(got[b] - want) <= tol, (b, got[b], want)


def test_metropolis_target_batch_against_oracle(engine):
    """Proposals of the Metropolis target shape (24 photons in 48 modes,
    occupations <= 4, Haar(48) seed 3) as one complex64 batch of 512; 64 of
    them against the oracle on the complex64-rounded matrix."""
    rng = np.random.default_rng(11)
    d, n = 48, 24
    U = haar_unitary(d, 3).astype(np.complex64)
    inp = np.array([1] * n + [0] * (d - n))
    R = []
    while len(R) < 512:
        r = np.bincount(rng.integers(0, d, n), minlength=d)
        if r.max() <= 4:
            R.append(r)
    R = np.stack(R)
    got = engine.permanent_batch(U, R, inp)
    U128 = U.astype(np.complex128)
    for b in range(0, 512, 8):
        want = oracle.permanent(U128, R[b], inp)
        tol = max(1e-5 * abs(want), 2.0 ** -23 * oracle.perm_abs(U128, R[b], inp))
        assert abs(complex(got[b]) - want) <= tol, (b, got[b], want)
