"""CPU tests of the Metropolis sampler's sample-quality estimate: the
integrated autocorrelation time against processes whose value is known in
closed form."""

import numpy as np

from piquasso_gb300.metropolis import chain_autocorrelation, integrated_autocorrelation


def test_independent_draws_have_unit_tau():
    rng = np.random.default_rng(0)
    assert abs(integrated_autocorrelation(rng.normal(size=(2000, 64))) - 1.0) < 0.05


def test_ar1_process():
    # x_t = phi x_{t-1} + e_t: tau = (1 + phi) / (1 - phi)
    rng = np.random.default_rng(1)
    phi = 0.5
    e = rng.normal(size=(4000, 64))
    x = np.zeros_like(e)
    for t in range(1, len(e)):
        x[t] = phi * x[t - 1] + e[t]
    assert abs(integrated_autocorrelation(x) - 3.0) < 0.15


def test_independence_chain_with_rejections():
    # an independence sampler that accepts with probability a keeps its state
    # otherwise: tau = (2 - a) / a for any statistic of the fresh draws
    rng = np.random.default_rng(2)
    a = 0.4
    cur = rng.normal(size=64)
    z = np.zeros((4000, 64))
    for t in range(len(z)):
        acc = rng.random(64) < a
        cur = np.where(acc, rng.normal(size=64), cur)
        z[t] = cur
    assert abs(integrated_autocorrelation(z) - (2 - a) / a) < 0.2


def test_chain_autocorrelation_reads_step_major_samples():
    # two modes: mode 0 repeats (tau 4), mode 1 is constant (tau 1)
    rng = np.random.default_rng(3)
    chains, steps = 32, 3000
    cur = rng.integers(0, 5, size=chains)
    S = np.zeros((steps, chains, 2), dtype=np.int64)
    for t in range(steps):
        acc = rng.random(chains) < 0.4
        cur = np.where(acc, rng.integers(0, 5, size=chains), cur)
        S[t, :, 0] = cur
        S[t, :, 1] = 3
    tmax, tmean = chain_autocorrelation(S.reshape(steps * chains, 2), chains)
    assert abs(tmax - 4.0) < 0.4
    assert abs(tmean - (tmax + 1.0) / 2) < 1e-12
