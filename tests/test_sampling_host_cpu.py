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


# --- the reference-RNG sampler's host logic (generate_samples: the lockstep
# photon steps and the vectorised pmf) against the reference's seeded goldens,
# its batched Laplace call answered by the oracle


@pytest.fixture
def rng_mode_on_cpu(monkeypatch):
    from piquasso_gb300 import sampling
    from test_postselect import _oracle_laplace_batch

    monkeypatch.setattr(sampling, "permanent_laplace_batch", _oracle_laplace_batch)
    return sampling


def test_seeded_golden_on_cpu(rng_mode_on_cpu):
    from conftest import as_matrix, load_golden

    g = load_golden("sampler_seeded.json")
    samples = rng_mode_on_cpu.generate_samples(g["input"], g["shots"], as_matrix(g["U"]), g["seed"], batch_size=7)
    assert [list(s) for s in samples] == g["generated_samples"]
    assert [list(s) for s in rng_mode_on_cpu.result_samples(samples, g["seed"])] == g["expected_samples"]


def test_seeded_lossy_goldens_on_cpu(rng_mode_on_cpu):
    from conftest import as_matrix, load_golden

    for c in load_golden("sampler_lossy_seeded.json")["cases"]:
        M = as_matrix(c["matrix"]).astype(np.complex128)
        got = rng_mode_on_cpu.sample(np.array(c["input"]), c["shots"], M, c["seed"])
        assert [list(s) for s in got] == c["generated_samples"], c["kind"]


def test_overlap_and_loss_match_restatement_on_cpu(rng_mode_on_cpu):
    from oracle import sampler as osampler

    U = haar_unitary(4, 8) * np.sqrt(0.8)
    inp = np.array([2, 1, 1, 0])
    got = rng_mode_on_cpu.generate_samples(inp, 40, U, 5, transmission=0.8, particle_overlap=0.6)
    want = osampler.generate_samples(inp, 40, oracle.permanent_laplace_dd, U, 5, transmission=0.8, overlap=0.6)
    assert got == want


def test_vectorised_pmf_matches_the_reference_loop():
    """sampling._pmf_batch against the oracle's per-shot restatement of the
    reference's _calculate_pmf (sampling.py:723-749; Python loops over modes
    on numpy scalars) for shots with different numbers of terms, repeated
    input modes and an empty output.  Array and scalar complex arithmetic in
    numpy differ in the last bits (6e-16 here), which the seeded goldens
    above never notice; the terms' order is the reference's."""
    from oracle import sampler as osampler
    from piquasso_gb300 import sampling

    d = 7
    U = haar_unitary(d, 12)
    rng = np.random.default_rng(3)
    cur, out = [], []
    for k in range(1, 8):
        c = np.bincount(rng.integers(0, d, k), minlength=d)
        o = np.bincount(rng.integers(0, d, k - 1), minlength=d)
        cur.append(c)
        out.append(o)
    cur, out = np.array(cur), np.array(out)
    lap = np.zeros((len(cur), d), dtype=np.complex128)
    want = []
    for s in range(len(cur)):
        if out[s].sum() > 0:
            lap[s] = oracle.permanent_laplace_dd(U, out[s], cur[s])[:d]
        nz = np.nonzero(cur[s])[0]

        def laplace(matrix, rows, cols, s=s, nz=nz):
            return np.array([1.0 + 0.0j]) if rows.sum() == 0 else lap[s][nz]

        want.append(osampler.calculate_pmf(cur[s], out[s], laplace, U))
    got = sampling._pmf_batch(U, cur, out, lap)
    want = np.array(want)
    assert np.max(np.abs(got - want) / want) < 1e-14


def test_draw_from_pmf_is_generator_choice():
    """One rng.random() per shot and a count over the normalised cumulative
    sum give what rng.choice(np.arange(d), p=pmf) gives, and leave every
    generator in the same state."""
    import copy

    from piquasso_gb300 import sampling

    master = np.random.default_rng(123)
    for trial in range(300):
        d = int(master.integers(2, 60))
        pmf = master.random((4, d)) ** 3 + 1e-300
        pmf[0, master.integers(0, d)] = 0.0
        pmf /= pmf.sum(axis=1, keepdims=True)
        gens = [np.random.default_rng(trial * 4 + s) for s in range(4)]
        twins = [copy.deepcopy(g) for g in gens]
        want = [g.choice(np.arange(d), p=pmf[s]) for s, g in enumerate(gens)]
        got = sampling._draw_from_pmf(pmf, np.array([g.random() for g in twins]))
        assert list(got) == want
        assert all(a.random() == b.random() for a, b in zip(gens, twins))
