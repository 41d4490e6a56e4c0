"""Exact boson sampling on the GPU (Clifford & Clifford algorithm B).

A drop-in for the lossless, indistinguishable path of the reference's
``PassiveSimulator`` sampler (piquasso/_simulators/passive/sampling.py:149-236,
711-753).  Every shot keeps its own ``np.random.default_rng(seed + idx)`` and
draws exactly the random numbers the reference draws, in the same order, so a
given seed reproduces the reference's samples.  What changes is the schedule:
all shots advance one photon at a time together, and each photon step is ONE
batched Laplace-permanent launch over every shot (``permanent_laplace_batch``)
instead of one CPU call per shot and step.

``result_samples`` reproduces ``Result.samples`` (piquasso/api/result.py:104-136):
the generated samples binned by first occurrence (piquasso/_utils.py:23-31),
expanded, then shuffled with ``random.Random(seed)``.
"""

import random

import numpy as np

from .permanent import permanent_laplace_batch


def to_first_quantized(occupation_numbers):
    occ = np.asarray(occupation_numbers)
    return np.repeat(np.arange(len(occ)), occ).astype(occ.dtype)


def _pmf_batch(U, current_input, samples, laplace):
    """pmf[s, idx] of sampling.py:723-749 for every shot, with the reference's
    summation order (over the nonzero input modes in increasing order, then the
    normalisation over idx in increasing order)."""
    shots, d = samples.shape
    pmf = np.empty((shots, d), dtype=np.float64)
    for s in range(shots):
        nz = np.nonzero(current_input[s] > 0)[0]
        if samples[s].sum() == 0:
            # empty output: the reference's Laplace vector is [1] (one entry)
            part = {nz[0]: 1.0 + 0.0j}
            terms = 1
        else:
            part = laplace[s]
            terms = len(nz)
        amp = np.zeros(d, dtype=np.complex128)
        for j in range(terms):
            amp = amp + (current_input[s, nz[j]] * part[nz[j]]) * U[:, nz[j]]
        p = np.abs(amp) ** 2
        norm = 0.0
        for idx in range(d):
            norm += p[idx]
        pmf[s] = p / norm
    return pmf


def generate_samples(input_state, shots, interferometer, seed, batch_size=4096):
    """Samples of the lossless boson sampler, as tuples, in generation order.

    ``input_state``: occupation numbers (length d); ``interferometer``: the
    d x d matrix (its dtype picks complex64 or complex128 permanents);
    ``seed``: the reference's ``config.seed_sequence`` (shot idx uses seed + idx).
    """
    U = np.asarray(interferometer)
    if U.dtype not in (np.complex64, np.complex128):
        U = U.astype(np.complex128)
    U128 = U.astype(np.complex128)
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    n = int(inp.sum())
    fq = to_first_quantized(inp)
    out = []
    for b0 in range(0, shots, batch_size):
        nb = min(batch_size, shots - b0)
        rngs = [np.random.default_rng(seed=seed + b0 + i) for i in range(nb)]
        samples = np.zeros((nb, d), dtype=int)
        current = np.zeros((nb, d), dtype=int)
        to_shrink = [np.copy(fq) for _ in range(nb)]
        for _ in range(1, n + 1):
            for s in range(nb):
                k = rngs[s].choice(len(to_shrink[s]))
                current[s, to_shrink[s][k]] += 1
                to_shrink[s] = np.delete(to_shrink[s], k)
            # Laplace permanents of every shot: rows = sample, cols = current input
            lap = permanent_laplace_batch(U, samples, current).astype(np.complex128)
            pmf = _pmf_batch(U128, current, samples, lap)
            for s in range(nb):
                idx = rngs[s].choice(np.arange(d), p=pmf[s])
                samples[s, idx] += 1
        out.extend(tuple(int(x) for x in row) for row in samples)
    return out


def get_counts(samples):
    counts = {}
    for s in samples:
        counts[s] = counts.get(s, 0) + 1
    return counts


def result_samples(samples, seed):
    """What the reference's ``Result.samples`` returns for these samples."""
    out = []
    for outcome, mult in get_counts(samples).items():
        out.extend([tuple(outcome)] * mult)
    random.Random(seed).shuffle(out)
    return out


def generate_samples_batched(input_state, shots, interferometer, seed, batch_size=2048, timings=None):
    """Exact samples of the same distribution, at throughput.

    Same algorithm (Clifford & Clifford B, sampling.py:208-236 of the
    reference): at step k a uniformly random not-yet-placed input photon joins
    the input, the conditional pmf over the d output modes comes from the
    Laplace permanents of (sample, current input), and one output mode is drawn.
    Differences from :func:`generate_samples`, all in the random-number
    plumbing: one generator drives all shots, the photon order is a random
    permutation drawn up front (equivalent to picking a uniformly random
    remaining photon at every step), and the pmf and the draw are vectorised
    over shots.  The samples therefore follow the reference's distribution but
    not its per-seed sequence.  Returns an int array (shots, d).

    ``timings`` (optional dict) receives the seconds spent in the batched
    Laplace calls ("laplace_s") and in total ("total_s").
    """
    import time

    t_start = time.perf_counter()
    U = np.asarray(interferometer)
    if U.dtype not in (np.complex64, np.complex128):
        U = U.astype(np.complex128)
    U128 = U.astype(np.complex128)
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    n = int(inp.sum())
    fq = to_first_quantized(inp)
    rng = np.random.default_rng(seed)
    out = np.zeros((shots, d), dtype=np.int64)
    t_lap = 0.0
    for b0 in range(0, shots, batch_size):
        nb = min(batch_size, shots - b0)
        order = np.argsort(rng.random((nb, n)), axis=1)
        photons = fq[order]  # (nb, n): the input mode joining at each step
        samples = np.zeros((nb, d), dtype=np.int64)
        current = np.zeros((nb, d), dtype=np.int64)
        rows = np.arange(nb)
        for k in range(n):
            current[rows, photons[:, k]] += 1
            if k == 0:
                # empty output: the Laplace vector is [1] at the only input column
                lap = np.zeros((nb, d), dtype=np.complex128)
                lap[rows, photons[:, 0]] = 1.0
            else:
                t0 = time.perf_counter()
                lap = permanent_laplace_batch(U, samples, current).astype(np.complex128)
                t_lap += time.perf_counter() - t0
            amp = (current * lap) @ U128.T  # amp[s, idx] = sum_j cur_j L_j U[idx, j]
            pmf = np.abs(amp) ** 2
            cdf = np.cumsum(pmf, axis=1)
            u = rng.random(nb) * cdf[:, -1]
            idx = np.minimum((cdf < u[:, None]).sum(axis=1), d - 1)
            samples[rows, idx] += 1
        out[b0:b0 + nb] = samples
    if timings is not None:
        timings["laplace_s"] = t_lap
        timings["total_s"] = time.perf_counter() - t_start
    return out
