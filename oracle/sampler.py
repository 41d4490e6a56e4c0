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


def generate_sample(d, n, permanent_laplace, interferometer, first_quantized_input, rng):
    sample = np.zeros(d, dtype=int)
    current_input = np.zeros(d, dtype=int)
    to_shrink = np.copy(first_quantized_input)
    for _ in range(1, n + 1):
        random_index = rng.choice(len(to_shrink))
        random_mode = to_shrink[random_index]
        current_input[random_mode] += 1
        to_shrink = np.delete(to_shrink, random_index)
        pmf = calculate_pmf(current_input, sample, permanent_laplace, interferometer)
        index = rng.choice(np.arange(pmf.shape[0]), p=pmf)
        sample[index] += 1
    return sample


def generate_samples(input_state, shots, permanent_laplace, interferometer, seed):
    input_state = np.asarray(input_state)
    d = len(input_state)
    n = int(np.sum(input_state))
    fq = to_first_quantized(input_state)
    out = []
    for idx in range(shots):
        rng = np.random.default_rng(seed=seed + idx)
        out.append(tuple(int(x) for x in generate_sample(d, n, permanent_laplace, interferometer, fq, rng)))
    return out


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
