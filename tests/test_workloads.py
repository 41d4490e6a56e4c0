"""CPU tests of the synthetic workload generators."""

import itertools

import numpy as np

from piquasso_gb300 import workloads


def test_haar_unitary_is_unitary_and_seeded():
    U = workloads.haar_unitary(12, 3)
    assert np.allclose(U @ U.conj().T, np.eye(12), atol=1e-12)
    assert np.array_equal(U, workloads.haar_unitary(12, 3))
    assert not np.array_equal(U, workloads.haar_unitary(12, 4))


def test_capped_compositions_are_uniform():
    n, d, cap = 4, 4, 2
    support = [c for c in itertools.product(range(cap + 1), repeat=d) if sum(c) == n]
    N = workloads.composition_counts(n, d, cap)
    assert N[d][n] == len(support)
    draws = workloads.capped_compositions(n, d, cap, 6000, seed=1)
    assert np.all(draws.sum(axis=1) == n) and draws.max() <= cap
    counts = {c: 0 for c in support}
    for row in draws:
        counts[tuple(int(x) for x in row)] += 1
    expected = len(draws) / len(support)
    chi2 = sum((c - expected) ** 2 / expected for c in counts.values())
    # 18 degrees of freedom: the 99.9% quantile is about 42.3
    assert chi2 < 42.3, chi2


def test_config_batch_patterns():
    P = workloads.capped_compositions(20, 40, 4, 64, seed=1)
    assert P.shape == (64, 40) and np.all(P.sum(axis=1) == 20) and P.max() <= 4
    steps = [workloads.gray_steps(p) for p in P]
    assert all(s >= 1 for s in steps)
