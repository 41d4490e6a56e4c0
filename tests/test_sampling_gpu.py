"""GPU exact sampler: reproduces the reference's seeded golden samples, and the
batched Laplace permanents it is built on match single calls and the oracle."""

import numpy as np
import pytest

import oracle
from conftest import as_matrix, haar_unitary, load_golden

pytestmark = pytest.mark.gpu


def test_gpu_sampler_reproduces_reference_golden(engine):
    from piquasso_gb300 import sampling

    g = load_golden("sampler_seeded.json")
    U = as_matrix(g["U"])
    samples = sampling.generate_samples(g["input"], g["shots"], U, g["seed"])
    assert [list(s) for s in samples] == g["generated_samples"]
    assert [list(s) for s in sampling.result_samples(samples, g["seed"])] == g["expected_samples"]


def test_gpu_sampler_small_batches_agree(engine):
    from piquasso_gb300 import sampling

    U = haar_unitary(8, 11)
    inp = [1, 1, 0, 2, 0, 1, 0, 0]
    a = sampling.generate_samples(inp, 30, U, 99, batch_size=7)
    b = sampling.generate_samples(inp, 30, U, 99, batch_size=64)
    assert a == b
    assert all(sum(s) == sum(inp) for s in a)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_laplace_batch_matches_oracle(engine, dtype):
    rng = np.random.default_rng(3)
    d = 10
    U = haar_unitary(d, 5).astype(dtype)
    B = 25
    R = np.zeros((B, d), dtype=int)
    C = np.zeros((B, d), dtype=int)
    for b in range(B):
        k = int(rng.integers(1, 9))
        C[b] = np.bincount(rng.choice(d, k, replace=False), minlength=d)
        R[b] = np.bincount(rng.integers(0, d, k - 1), minlength=d)
    got = engine.permanent_laplace_batch(U, R, C)
    for b in range(B):
        want = oracle.permanent_laplace_dd(U.astype(np.complex128), R[b], C[b])
        if R[b].sum() == 0:
            assert got[b, 0] == 1 and np.all(got[b, 1:] == 0)
            continue
        nz = C[b] > 0
        rt = 1e-4 if dtype == np.complex64 else 1e-10
        assert np.allclose(got[b][nz], want[nz], rtol=rt, atol=rt * 1e-3), b


def test_batched_sampler_matches_exact_marginals(engine):
    """The throughput sampler draws from the exact distribution: its one- and
    two-mode marginals agree with the binomial-moment marginals to within the
    sampling noise of 20000 samples."""
    from piquasso_gb300 import marginals, sampling

    d, n = 8, 4
    U = haar_unitary(d, 31)
    inp = [1] * n + [0] * (d - n)
    S = sampling.generate_samples_batched(inp, 20000, U, seed=5)
    assert S.shape == (20000, d) and np.all(S.sum(axis=1) == n)
    tv2 = marginals.tvd_two_mode(S, inp, U, [(0, 1), (2, 7), (5, 6)])
    tv1 = marginals.tvd_one_mode(S, inp, U, range(d))
    assert np.all(tv2 < 0.02), tv2
    assert np.all(tv1 < 0.015), tv1


def _numpy_step(engine, U, R, C, u):
    """The unfused step: batched Laplace permanents, then the pmf and the
    inverse-CDF draw of the reference's sampling loop in numpy."""
    lap = engine.permanent_laplace_batch(U, R, C).astype(np.complex128)
    amp = (C * lap) @ U.astype(np.complex128).T
    cdf = np.cumsum(np.abs(amp) ** 2, axis=1)
    return np.minimum((cdf < (u * cdf[:, -1])[:, None]).sum(axis=1), U.shape[0] - 1)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_fused_sampler_step_matches_unfused(engine, dtype):
    rng = np.random.default_rng(17)
    d = 16
    U = haar_unitary(d, 8).astype(dtype)
    B = 400
    R = np.zeros((B, d), dtype=int)
    C = np.zeros((B, d), dtype=int)
    for b in range(B):
        k = int(rng.integers(2, 11))
        C[b] = np.bincount(rng.integers(0, d, k), minlength=d)  # repeated input photons too
        R[b] = np.bincount(rng.integers(0, d, k - 1), minlength=d)
    u = rng.random(B)
    got = engine.sampler_step_batch(U, R, C, u)
    want = _numpy_step(engine, U, R, C, u)
    assert got.dtype == np.int64 and got.shape == (B,)
    assert np.array_equal(got, want)
    # the draw's edges: u = 0 takes mode 0, u just below 1 the last mode of
    # nonzero probability
    got0 = engine.sampler_step_batch(U, R[:50], C[:50], np.zeros(50))
    assert np.array_equal(got0, _numpy_step(engine, U, R[:50], C[:50], np.zeros(50)))
    u1 = np.full(50, np.nextafter(1.0, 0.0))
    assert np.array_equal(engine.sampler_step_batch(U, R[:50], C[:50], u1), _numpy_step(engine, U, R[:50], C[:50], u1))


def test_fused_sampler_step_rejects_empty_shots(engine):
    d = 6
    U = haar_unitary(d, 2)
    R = np.zeros((2, d), dtype=int)
    C = np.zeros((2, d), dtype=int)
    R[0, 1] = 1
    C[0, :2] = 1
    C[1, 0] = 1  # shot 1 has no output photon yet
    with pytest.raises(engine.PermanentInputError):
        engine.sampler_step_batch(U, R, C, np.full(2, 0.5))
    assert len(engine.sampler_step_batch(U, R[:0], C[:0], np.zeros(0))) == 0


def test_fused_sampler_step_many_modes(engine):
    """More output modes than a warp takes at once (several chunks of 32)."""
    rng = np.random.default_rng(4)
    d = 100
    U = haar_unitary(d, 12)
    B = 64
    R = np.zeros((B, d), dtype=int)
    C = np.zeros((B, d), dtype=int)
    for b in range(B):
        C[b] = np.bincount(rng.choice(d, 6, replace=False), minlength=d)
        R[b] = np.bincount(rng.integers(0, d, 5), minlength=d)
    u = rng.random(B)
    assert np.array_equal(engine.sampler_step_batch(U, R, C, u), _numpy_step(engine, U, R, C, u))
