"""Seeded synthetic inputs for the permanent and boson-sampling workloads.

* :func:`haar_unitary` — a Haar-random unitary: QR of a complex Gaussian
  matrix with the phase fix U = Q diag(r_ii / |r_ii|).
* :func:`capped_compositions` — output patterns drawn uniformly from the weak
  compositions of n into d parts with every part at most ``cap``: the number
  of completions is counted by dynamic programming and each part is drawn in
  turn with probability proportional to the completions it leaves, so every
  pattern is equally likely (an exact sampler, unlike rejection from
  multinomial draws, which is not uniform).
"""

import numpy as np


def haar_unitary(d, seed):
    rng = np.random.default_rng(seed)
    Z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    Q, R = np.linalg.qr(Z)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


def composition_counts(n, d, cap):
    """N[k][r]: weak compositions of r into k parts, each part in [0, cap]
    (exact Python integers)."""
    N = [[0] * (n + 1) for _ in range(d + 1)]
    N[0][0] = 1
    for k in range(1, d + 1):
        for r in range(n + 1):
            N[k][r] = sum(N[k - 1][r - v] for v in range(0, min(cap, r) + 1))
    return N


def capped_compositions(n, d, cap, count, seed):
    """``count`` patterns (shape (count, d), int) uniform over the weak
    compositions of n into d parts with parts <= cap."""
    N = composition_counts(n, d, cap)
    if N[d][n] == 0:
        raise ValueError("no composition of %d into %d parts of at most %d" % (n, d, cap))
    rng = np.random.default_rng(seed)
    out = np.zeros((count, d), dtype=np.int64)
    for s in range(count):
        r = n
        for i in range(d):
            k = d - i - 1  # parts left after this one
            total = N[k + 1][r]
            # uniform integer in [0, total) from 64-bit draws (total < 2^64 here)
            u = int(rng.integers(0, 2 ** 62)) * (2 ** 62) + int(rng.integers(0, 2 ** 62))
            u %= total
            for v in range(0, min(cap, r) + 1):
                c = N[k][r - v]
                if u < c:
                    out[s, i] = v
                    r -= v
                    break
                u -= c
    return out


def gray_steps(rows):
    """Gray-code steps of one permanent with these row multiplicities after the
    reference's reduction (one copy of a smallest nonzero row split off):
    prod over rows of (m_i + 1), with m reduced by one at that row."""
    rows = np.asarray(rows, dtype=np.int64)
    nz = rows[rows > 0]
    if nz.size == 0:
        return 0
    m = rows.copy()
    idx = int(np.flatnonzero(rows == nz.min())[0])
    m[idx] -= 1
    return int(np.prod(m[m > 0] + 1))
