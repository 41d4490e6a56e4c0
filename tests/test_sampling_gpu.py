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
