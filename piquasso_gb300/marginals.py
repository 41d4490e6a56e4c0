"""Exact marginal probabilities of ideal boson sampling on the GPU, the
marginal sampler, and the total-variation judge of the samplers.

The method of the reference's piquasso/_simulators/passive/marginal.py
(low-rank marginal generating function, lines 15-92): for the selected output
modes T and every occupied input mode a with r_a photons, with
f_a(z) = sum_j conj(U[T_j, a]) z_j,

    P(z, w) = prod_a L_{r_a}(-f_a(z) conj(f_a(w)))

has diagonal coefficients whose scaled values b_alpha = alpha! P_{alpha,alpha}
are the binomial moments E[prod_j C(X_j, alpha_j)] of the output photon
numbers on T; the probabilities follow by the binomial transform

    Pr(X = y) = sum_{alpha >= y} b_alpha prod_j C(alpha_j, y_j) (-1)^(alpha_j - y_j).

The moments come from the engine's GPU dynamic program
(``pqg_binomial_moments_c128``: degree blocks of P, two gather launches per
input mode, many mode sets per call); the transform runs on the host over the
(n+1)^k moments.
"""

import ctypes
from math import comb

import numpy as np

from . import _lib


def binomial_moments_sets(input_photons, U, mode_sets, max_device_bytes=0):
    """Binomial moments of every mode set (all of the same size k): array
    (n_sets,) + (n+1,)*k, b[alpha] = E[prod_j C(X_j, alpha_j)] (0 where
    |alpha| > n)."""
    inp = np.ascontiguousarray(np.asarray(input_photons).astype(np.int32))
    Uc = np.ascontiguousarray(np.asarray(U, dtype=np.complex128))
    M = np.ascontiguousarray(np.atleast_2d(np.asarray(mode_sets)).astype(np.int32))
    n_sets, k = M.shape
    d = len(inp)
    if Uc.shape != (d, d):
        raise ValueError("the interferometer must be %d x %d" % (d, d))
    n = int(inp.sum())
    out = np.zeros((n_sets,) + (n + 1,) * k, dtype=np.float64)
    L = _lib.load()
    st = L.pqg_binomial_moments_c128(Uc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), d,
                                     inp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                     M.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), k, n_sets,
                                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(max_device_bytes))
    if st:
        from .permanent import _raise_for

        _raise_for(st)
    return out


def binomial_moments(input_photons, U, modes):
    """b[alpha] for alpha over {0..n}^k, k = len(modes)."""
    return binomial_moments_sets(input_photons, U, [tuple(modes)])[0]


def _transform(b):
    """Pr(X = y) from the binomial moments, one axis at a time:
    M[y, alpha] = C(alpha, y) (-1)^(alpha - y)."""
    n = b.shape[-1] - 1
    T = np.zeros((n + 1, n + 1))
    for y in range(n + 1):
        for al in range(y, n + 1):
            T[y, al] = comb(al, y) * (-1) ** (al - y)
    p = b
    for ax in range(1, b.ndim):
        p = np.moveaxis(np.tensordot(T, np.moveaxis(p, ax, 0), axes=(1, 0)), 0, ax)
    return np.clip(p, 0.0, None)


def marginals(input_photons, U, mode_sets):
    """Pr(X_T = y) for every mode set T: array (n_sets,) + (n+1,)*k."""
    return _transform(binomial_moments_sets(input_photons, U, mode_sets))


def marginal(input_photons, U, modes):
    """Pr(X_T = y) as an array over y in {0..n}^k, k = len(modes)."""
    return marginals(input_photons, U, [tuple(modes)])[0]


def get_marginal_fock_probabilities(input_photons, U, postselected_modes, postselected_photons, marginal_modes):
    """The reference's get_marginal_fock_probabilities (marginal.py:103-160):
    {outcome on marginal_modes: joint probability with the postselection}
    over every outcome with at most n - sum(postselected_photons) photons."""
    post = tuple(int(m) for m in postselected_modes)
    photons = tuple(int(x) for x in postselected_photons)
    modes = post + tuple(int(m) for m in marginal_modes)
    n = int(np.sum(input_photons))
    p = marginal(input_photons, U, modes)[photons] if post else marginal(input_photons, U, modes)
    left = n - sum(photons)
    out = {}
    for y in np.ndindex(*((left + 1,) * len(marginal_modes))):
        if sum(y) <= left:
            out[tuple(int(v) for v in y)] = float(p[y])
    return out


def generate_marginal_samples(input_photons, U, modes, shots, seed, postselected_modes=(),
                              postselected_photons=()):
    """Samples of the output photon numbers on `modes` only, drawn mode by
    mode from the exact conditional marginals (the reference's
    generate_marginal_samples, sampling.py:796-857): for every mode a uniform
    threshold from ``np.random.default_rng(seed)`` and the smallest photon
    number whose cumulative conditional probability reaches it."""
    n = int(np.sum(input_photons))
    post = tuple(postselected_modes)
    pp = np.asarray(postselected_photons, dtype=int)
    k = len(modes)
    joint = marginal(input_photons, U, post + tuple(modes))  # over (post, modes)
    if post:
        joint = joint[tuple(pp)]
    left = n - int(pp.sum())
    # prefix marginals: pref[i][y_0..y_i] = Pr(post, Y_0..Y_i = y_0..y_i)
    pref = [None] * k
    acc = joint
    for i in range(k - 1, -1, -1):
        pref[i] = acc
        acc = acc.sum(axis=-1)
    total = float(acc) if np.ndim(acc) == 0 else float(np.sum(acc))
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(shots):
        prev = total
        y = []
        rem = left
        for i in range(k):
            thr = rng.random()
            cum = 0.0
            row = pref[i][tuple(y)]
            for t in range(rem + 1):
                p = float(row[t])
                cum += p / prev if prev > 0 else 0.0
                if cum >= thr:
                    break
            y.append(t)
            rem -= t
            prev = float(row[t])
        out.append(tuple(y))
    return out


def empirical_two_mode(samples, modes, n):
    S = np.asarray(samples)
    h = np.zeros((n + 1, n + 1))
    np.add.at(h, (S[:, modes[0]], S[:, modes[1]]), 1.0)
    return h / len(S)


def tvd_two_mode(samples, input_photons, U, pairs):
    """Total-variation distance of the samples' two-mode marginals from the
    exact ones, per pair of modes: 0.5 * sum |p_exact - p_empirical|."""
    n = int(np.sum(input_photons))
    ex = marginals(input_photons, U, [tuple(p) for p in pairs])
    out = []
    for i, pair in enumerate(pairs):
        em = empirical_two_mode(samples, pair, n)
        out.append(0.5 * float(np.abs(ex[i] - em).sum()))
    return np.array(out)


def tvd_one_mode(samples, input_photons, U, modes):
    n = int(np.sum(input_photons))
    S = np.asarray(samples)
    ex = marginals(input_photons, U, [(m,) for m in modes])
    out = []
    for i, m in enumerate(modes):
        em = np.bincount(S[:, m], minlength=n + 1)[: n + 1] / len(S)
        out.append(0.5 * float(np.abs(ex[i] - em).sum()))
    return np.array(out)
