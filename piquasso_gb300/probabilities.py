"""Exact output probabilities of ideal boson sampling, batched on the GPU, and
linear cross-entropy (LXEB) scoring of sample sets.

``detection_probabilities`` is the batched form of the reference's
``PassiveState.get_particle_detection_probability`` for lossless,
indistinguishable photons (piquasso/_simulators/passive/state.py:292-361 →
probabilities.py:26-54 ``get_ideal_particle_number_probability`` →
utils.py:131-138 ``calculate_inner_product``): for a state
sum_k c_k |x_k> and an output pattern y,

    p(y) = | sum_{k: |x_k| = |y|} c_k perm(U; rows=y, cols=x_k) / sqrt(prod y! prod x_k!) |^2 .

Every input occupation x_k costs ONE batched permanent launch over all the
output patterns (``permanent_batch``), instead of one CPU call per pattern.

``lxe_ref_boson_sampling`` is the Haar-averaged LXEB reference value of boson
sampling with n photons in m modes — E_U[sum_y p_U(y)^2], the expected mean
ideal probability of ideally drawn samples — from the closed form of
arXiv:2604.15258 (the reference's piquasso/lxeb.py:66-106), evaluated as a
log-sum-exp.  ``lxeb_score`` averages the ideal probabilities of a sample set
and normalises by that reference value (about 1 for an ideal sampler on a
typical Haar interferometer).
"""

import math

import numpy as np

from .permanent import permanent_batch


def _log_factorials(kmax):
    return np.array([math.lgamma(k + 1.0) for k in range(kmax + 1)])


def detection_probabilities(interferometer, outputs, inputs, coefficients=None, mode="auto"):
    """Ideal detection probabilities of many output patterns.

    ``outputs``: (B, d) occupation numbers; ``inputs``: one occupation vector
    (d,) or several (K, d) with ``coefficients`` (K,) (default: 1 for a single
    input).  Returns a float64 array (B,).  The interferometer's dtype picks
    complex64 or complex128 permanents (``mode`` as for permanent_batch).
    """
    U = np.asarray(interferometer)
    Y = np.atleast_2d(np.asarray(outputs)).astype(np.int64)
    X = np.atleast_2d(np.asarray(inputs)).astype(np.int64)
    if coefficients is None:
        if len(X) != 1:
            raise ValueError("several input occupations need coefficients")
        coefficients = np.ones(1)
    c = np.asarray(coefficients, dtype=np.complex128).reshape(-1)
    if len(c) != len(X):
        raise ValueError("one coefficient per input occupation")
    if Y.shape[1] != U.shape[0] or X.shape[1] != U.shape[1]:
        raise ValueError("patterns must match the interferometer's modes")
    ny = Y.sum(axis=1)
    lf = _log_factorials(int(max(Y.max(initial=0), X.max(initial=0))))
    log_ny = lf[Y].sum(axis=1)
    amp = np.zeros(len(Y), dtype=np.complex128)
    for k, x in enumerate(X):
        sel = np.nonzero(ny == x.sum())[0]
        if len(sel) == 0:
            continue
        perms = permanent_batch(U, Y[sel], x, mode=mode).astype(np.complex128)
        amp[sel] += c[k] * perms * np.exp(-0.5 * (log_ny[sel] + lf[x].sum()))
    return np.abs(amp) ** 2


def get_particle_detection_probability(interferometer, occupation_number, inputs, coefficients=None):
    """One pattern: the reference's get_ideal_particle_number_probability."""
    return float(detection_probabilities(interferometer, [occupation_number], inputs, coefficients)[0])


def lxe_ref_boson_sampling(n, m):
    """Haar average of sum_y p(y)^2 for n photons in m modes (arXiv:2604.15258):

        2^n n! sum_{r=0}^{n//2} (2n-4r+1)/(2n-2r+1) 16^-r C(2r, r) / C(2n-2r, n-r)
                                  / ((m/2)_r ((m+1)/2)_(n-r))

    with (a)_k the rising Pochhammer symbol.  TypeError for non-integer
    arguments, ValueError for n < 0 or m < 1 (as the reference's function)."""
    if not isinstance(n, int) or not isinstance(m, int) or isinstance(n, bool) or isinstance(m, bool):
        raise TypeError("n and m must be integers")
    if n < 0:
        raise ValueError("n must be non-negative")
    if m <= 0:
        raise ValueError("m must be positive")

    def log_binom(a, b):
        return math.lgamma(a + 1) - math.lgamma(b + 1) - math.lgamma(a - b + 1)

    def log_rising(a, k):
        return 0.0 if k == 0 else math.lgamma(a + k) - math.lgamma(a)

    logs = []
    for r in range(n // 2 + 1):
        logs.append(math.log(2 * n - 4 * r + 1) - math.log(2 * n - 2 * r + 1) - r * math.log(16.0)
                    + log_binom(2 * r, r) - log_binom(2 * n - 2 * r, n - r)
                    - log_rising(m / 2.0, r) - log_rising((m + 1) / 2.0, n - r))
    top = max(logs)
    lse = top + math.log(sum(math.exp(v - top) for v in logs))
    return math.exp(n * math.log(2.0) + math.lgamma(n + 1) + lse)


def lxeb_score(interferometer, input_state, samples, mode="auto"):
    """Mean ideal probability of the samples, the Haar reference value and
    their ratio (``normalized``, about 1 for an ideal sampler)."""
    x = np.asarray(input_state).astype(np.int64)
    S = np.atleast_2d(np.asarray(samples)).astype(np.int64)
    p = detection_probabilities(interferometer, S, x, mode=mode)
    ref = lxe_ref_boson_sampling(int(x.sum()), int(len(x)))
    mean = float(p.mean()) if len(p) else 0.0
    return {"mean_probability": mean, "reference": ref, "normalized": mean / ref if ref > 0 else float("nan"),
            "samples": int(len(S))}
