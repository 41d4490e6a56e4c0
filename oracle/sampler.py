"""Numpy restatement of piquasso's exact boson sampler — TEST INFRASTRUCTURE ONLY.

Clifford & Clifford algorithm B (arXiv:1706.01260) as the reference implements
it for the lossless, indistinguishable case (reference paths, piquasso 8.0.1):
  * _generate_samples:   piquasso/_simulators/passive/sampling.py:149-194
    (one ``np.random.default_rng(seed + idx)`` per shot)
  * _grow_current_input: sampling.py:197-205
  * _generate_sample:    sampling.py:208-236
  * _filter_zeros:       sampling.py:711-720
  * _calculate_pmf:      sampling.py:723-749
  * _sample_from_pmf:    sampling.py:752-753
  * to_first_quantized:  piquasso/_math/indices.py:104-114
  * result_samples:      piquasso/_utils.py:23-31 (get_counts) and
    piquasso/api/result.py:104-136 (Result.samples: expand the binned counts,
    then shuffle them with random.Random(seed))
and the lossy and partially distinguishable variants that reuse the same
per-shot generator:
  * uniform loss: the reject condition ``config.rng.uniform() > s_0^2`` drawn
    once per photon step from the configuration's generator
    (np.random.default_rng(seed)), passive/simulation_steps.py:342-362;
  * uniform particle overlap: _generate_sample_with_uniform_overlap,
    _separate_particles, _sample_distinguishable_particles (sampling.py:328-418);
  * non-uniform loss: generate_lossy_samples and the SVD dilation into 2d
    modes (sampling.py:110-146, 756-784).
The Laplace permanents come from the function passed in, so the same
restatement runs on the reference's compiled module, on the double-double
oracle, or on the GPU engine under test.  The random-number calls and their
order are those of the reference, so equal inputs and seeds give equal samples.
"""

import random

import numpy as np


def to_first_quantized(occupation_numbers):
    occ = np.asarray(occupation_numbers)
    return np.repeat(np.arange(len(occ)), occ).astype(occ.dtype)


def _filter_zeros(matrix, input_state, output_state):
    nz_in = input_state > 0
    nz_out = output_state > 0
    return matrix[np.ix_(nz_out, nz_in)], input_state[nz_in], output_state[nz_out]


def calculate_pmf(input_state, sample, permanent_laplace, interferometer):
    d = len(sample)
    nonzero_indices = np.arange(d)[input_state > 0]
    fU, fin, fout = _filter_zeros(interferometer, input_state, sample)
    partial = permanent_laplace(fU, fout, fin)
    pmf = np.empty(d, dtype=np.float64)
    normalization = 0.0
    for idx in range(d):
        perm = 0.0
        for j in range(len(partial)):
            perm += input_state[nonzero_indices[j]] * partial[j] * interferometer[idx, nonzero_indices[j]]
        pmf[idx] = np.abs(perm) ** 2
        normalization += pmf[idx]
    return pmf / normalization


def generate_sample(d, n, permanent_laplace, interferometer, first_quantized_input, rng, reject=None):
    sample = np.zeros(d, dtype=int)
    current_input = np.zeros(d, dtype=int)
    to_shrink = np.copy(first_quantized_input)
    for _ in range(1, n + 1):
        if reject is not None and reject():
            continue
        random_index = rng.choice(len(to_shrink))
        random_mode = to_shrink[random_index]
        current_input[random_mode] += 1
        to_shrink = np.delete(to_shrink, random_index)
        pmf = calculate_pmf(current_input, sample, permanent_laplace, interferometer)
        index = rng.choice(np.arange(pmf.shape[0]), p=pmf)
        sample[index] += 1
    return sample


def separate_particles(input_occupation, overlap, rng):
    from scipy.special import comb, factorial

    d = len(input_occupation)
    indist = np.zeros(d, dtype=int)
    dist = np.zeros(d, dtype=int)
    for j, n_j in enumerate(input_occupation):
        if n_j == 0:
            continue
        weights = np.array([comb(n_j, k) * (overlap ** k) * ((1.0 - overlap) ** (n_j - k)) * factorial(k)
                            for k in range(n_j + 1)], dtype=float)
        K = rng.choice(n_j + 1, p=weights / weights.sum())
        indist[j] = K
        dist[j] = n_j - K
    return indist, dist


def sample_distinguishable(interferometer, particles, rng, reject):
    d = len(particles)
    out = np.zeros(d, dtype=int)
    for mode, count in enumerate(particles):
        p = np.abs(interferometer[:, mode]) ** 2
        p = p / np.sum(p)
        for _ in range(count):
            o = rng.choice(d, p=p)
            if not reject():
                out[o] += 1
    return out


def generate_samples(input_state, shots, permanent_laplace, interferometer, seed, transmission=None, overlap=None):
    """``transmission``: uniform loss (photon kept with this probability,
    decided by the configuration generator); ``overlap``: uniform particle
    overlap of partially distinguishable photons."""
    input_state = np.asarray(input_state)
    d = len(input_state)
    n = int(np.sum(input_state))
    fq = to_first_quantized(input_state)
    config_rng = np.random.default_rng(seed)
    if transmission is None:
        reject = lambda: False  # noqa: E731
    else:
        reject = lambda: config_rng.uniform() > transmission  # noqa: E731
    out = []
    for idx in range(shots):
        rng = np.random.default_rng(seed=seed + idx)
        if overlap is None:
            s = generate_sample(d, n, permanent_laplace, interferometer, fq, rng, reject)
        else:
            indist, dist = separate_particles(input_state, overlap, rng)
            dist_out = sample_distinguishable(interferometer, dist, rng, reject)
            s = dist_out + generate_sample(d, int(indist.sum()), permanent_laplace, interferometer,
                                           to_first_quantized(indist), rng, reject)
        out.append(tuple(int(x) for x in s))
    return out


def expanded_interferometer(matrix):
    """The 2d x 2d dilation (first d columns orthonormal) of a lossy d x d matrix from its SVD
    M = V diag(s) W: blockdiag(V, I) [[diag s, diag c], [diag c, diag s]]
    blockdiag(W, I), c = sqrt(1 - s^2)."""
    V, sv, W = np.linalg.svd(matrix)
    d = len(sv)
    Z, I = np.zeros((d, d)), np.eye(d)
    c = np.diag(np.sqrt(1.0 - sv ** 2))
    EV = np.block([[V, Z], [Z, I]])
    EW = np.block([[W, Z], [Z, I]])
    S = np.block([[np.diag(sv), c], [c, np.diag(sv)]])
    return EV @ S @ EW


def generate_lossy_samples(input_state, shots, permanent_laplace, matrix, seed):
    """Non-uniform loss: the lossless sampler on the dilation, state padded
    with d empty modes, samples trimmed back to the first d modes."""
    input_state = np.asarray(input_state)
    d = len(input_state)
    expanded = expanded_interferometer(matrix)
    state = np.concatenate([input_state, np.zeros(d, dtype=input_state.dtype)])
    return [s[:d] for s in generate_samples(state, shots, permanent_laplace, expanded, seed)]


def get_counts(samples):
    counts = {}
    for s in samples:
        counts[s] = counts.get(s, 0) + 1
    return counts


def result_samples(samples, seed):
    """What ``Result.samples`` returns for these generated samples."""
    out = []
    for outcome, mult in get_counts(samples).items():
        out.extend([tuple(outcome)] * mult)
    random.Random(seed).shuffle(out)
    return out
