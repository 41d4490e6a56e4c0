"""The batched sampler's host logic on CPU: piquasso_gb300.sampling's
generate_samples_batched with its one engine call per photon step
(sampler_step_batch) replaced by the same step in numpy on the oracle's
double-double Laplace permanents.  Checks the photon bookkeeping (the random
photon order, the numpy first step, uniform loss, partial
distinguishability) and the distribution: one-mode marginals against the
exact marginals of the oracle's dynamic program."""

import numpy as np
import pytest

import oracle
from conftest import haar_unitary
from oracle import marginals as omarg


def _numpy_step(U, rows, cols, uniforms):
    """sampler_step_batch restated: Laplace permanents (oracle), the pmf
    |sum_j cols_j L_j U[i, j]|^2 and the inverse-CDF draw."""
    U = np.asarray(U, dtype=np.complex128)
    d = U.shape[0]
    modes = np.zeros(len(rows), dtype=np.int64)
    for s, (r, c, u) in enumerate(zip(rows, cols, uniforms)):
        assert r.sum() > 0 and c.sum() > 0
        lap = oracle.permanent_laplace_dd(U, r, c)
        amp = (c * lap[:d]) @ U.T
        cdf = np.cumsum(np.abs(amp) ** 2)
        modes[s] = min(int((cdf < u * cdf[-1]).sum()), d - 1)
    return modes


@pytest.fixture
def sampling_on_cpu(monkeypatch):
    from piquasso_gb300 import sampling

    monkeypatch.setattr(sampling, "sampler_step_batch", _numpy_step)
    return sampling


def _one_mode_tvd(S, inp, U):
    n = int(np.sum(inp))
    worst = 0.0
    for m in range(len(inp)):
        exact = omarg.marginal(inp, U, [m])
        emp = np.bincount(S[:, m], minlength=n + 1)[: n + 1] / len(S)
        worst = max(worst, 0.5 * float(np.abs(emp - exact).sum()))
    return worst


def test_lossless_counts_and_marginals(sampling_on_cpu):
    d = 6
    U = haar_unitary(d, 4)
    inp = np.array([1, 1, 0, 1, 0, 0])
    S = sampling_on_cpu.generate_samples_batched(inp, 3000, U, seed=9, batch_size=1000, workers=1)
    assert S.shape == (3000, d)
    assert np.all(S.sum(axis=1) == 3)
    assert _one_mode_tvd(S, inp, U) < 0.04


def test_multiphoton_inputs(sampling_on_cpu):
    d = 5
    U = haar_unitary(d, 6)
    inp = np.array([2, 0, 1, 0, 0])
    S = sampling_on_cpu.generate_samples_batched(inp, 3000, U, seed=3, batch_size=1500, workers=2)
    assert np.all(S.sum(axis=1) == 3)
    assert _one_mode_tvd(S, inp, U) < 0.04


def test_uniform_loss_keeps_a_binomial_number(sampling_on_cpu):
    d = 6
    U = haar_unitary(d, 8)
    inp = np.array([1, 1, 1, 1, 0, 0])
    S = sampling_on_cpu.generate_samples_batched(inp, 4000, U, seed=1, batch_size=2000, workers=1,
                                                transmission=0.5)
    counts = np.bincount(S.sum(axis=1), minlength=5)
    expect = np.array([1, 4, 6, 4, 1]) / 16.0
    assert 0.5 * np.abs(counts / len(S) - expect).sum() < 0.03


def test_distinguishable_photons_land_independently(sampling_on_cpu):
    """Overlap 0: every photon is distinguishable, so each lands by
    |U[:, j]|^2 on its own; the one-mode means are the sums of those columns."""
    d = 5
    U = haar_unitary(d, 2)
    inp = np.array([1, 1, 1, 0, 0])
    S = sampling_on_cpu.generate_samples_batched(inp, 4000, U, seed=5, batch_size=2000, workers=1,
                                                particle_overlap=0.0)
    assert np.all(S.sum(axis=1) == 3)
    means = (np.abs(U[:, :3]) ** 2).sum(axis=1)
    assert np.max(np.abs(S.mean(axis=0) - means)) < 0.05


def test_same_seed_same_samples(sampling_on_cpu):
    d = 5
    U = haar_unitary(d, 3)
    inp = np.array([1, 0, 1, 0, 1])
    a = sampling_on_cpu.generate_samples_batched(inp, 200, U, seed=11, batch_size=64, workers=1)
    b = sampling_on_cpu.generate_samples_batched(inp, 200, U, seed=11, batch_size=64, workers=3)
    assert np.array_equal(a, b)  # per-batch generators: the thread count does not matter
