"""CPU restatement of the exact one- and two-mode marginals — TEST
INFRASTRUCTURE ONLY (the checker of piquasso_gb300.marginals, which runs the
same dynamic program on the GPU for any number of modes).

The method of the reference's piquasso/_simulators/passive/marginal.py:15-92
(low-rank marginal generating function): for the selected output modes T and
every occupied input mode a with r_a photons, let f_a(z) = sum_j conj(U[T_j, a])
z_j.  The polynomial

    P(z, w) = prod_a L_{r_a}(-f_a(z) conj(f_a(w)))

(L_r the Laguerre polynomial) has diagonal coefficients P_{alpha,alpha} whose
scaled values b_alpha = alpha! P_{alpha,alpha} are the binomial moments
E[prod_j binom(X_j, alpha_j)] of the output photon numbers on T, and

    Pr(X = y) = sum_{alpha >= y} b_alpha prod_j binom(alpha_j, y_j) (-1)^(alpha_j - y_j).

Here the product is a dense dynamic program over the input modes on the
coefficient array indexed by (z-degrees, w-degrees), written for one and two
modes in numpy (the reference uses numba, which is not a dependency here).
"""

import itertools
from math import comb, factorial

import numpy as np


def _laguerre_terms(r):
    """L_r(-x) = sum_k binom(r, k) x^k / k!  ->  coefficients c_k for x^k."""
    return [comb(r, k) / factorial(k) for k in range(r + 1)]


def binomial_moments(input_photons, U, modes):
    """b[alpha] for alpha over {0..n}^k (k = len(modes), 1 or 2)."""
    inp = np.asarray(input_photons, dtype=int)
    U = np.asarray(U, dtype=np.complex128)
    n = int(inp.sum())
    k = len(modes)
    if k not in (1, 2):
        raise ValueError("one or two modes")
    D = n + 1
    # C[z-degrees..., w-degrees...]
    shape = (D,) * (2 * k)
    C = np.zeros(shape, dtype=np.complex128)
    C[(0,) * (2 * k)] = 1.0
    for a in np.nonzero(inp)[0]:
        r = int(inp[a])
        V = np.conj(U[list(modes), a])  # f_a(z) = sum_j V_j z_j
        # monomials of f(z) conj(f(w)): z_i w_j with coefficient V_i conj(V_j)
        bil = [((i, j), V[i] * np.conj(V[j])) for i in range(k) for j in range(k)]
        # power series of the factor: sum_m c_m (f conj f)^m
        new = np.zeros_like(C)
        term = C.copy()
        for m, cm in enumerate(_laguerre_terms(r)):
            if m > 0:
                nxt = np.zeros_like(C)
                for (i, j), coef in bil:
                    sl_src = [slice(None)] * (2 * k)
                    sl_dst = [slice(None)] * (2 * k)
                    sl_src[i] = slice(0, D - 1)
                    sl_dst[i] = slice(1, D)
                    sl_src[k + j] = slice(0, D - 1)
                    sl_dst[k + j] = slice(1, D)
                    nxt[tuple(sl_dst)] += coef * term[tuple(sl_src)]
                term = nxt
            new += cm * term
        C = new
    b = np.zeros((D,) * k)
    for alpha in itertools.product(range(D), repeat=k):
        if sum(alpha) > n:
            continue
        b[alpha] = np.real(C[alpha + alpha]) * np.prod([factorial(x) for x in alpha])
    return b


def marginal(input_photons, U, modes):
    """Pr(X_T = y) as an array over y in {0..n}^k (k = 1 or 2)."""
    b = binomial_moments(input_photons, U, modes)
    n = b.shape[0] - 1
    k = b.ndim
    # binomial transform, one axis at a time: M[y, alpha] = binom(alpha, y)(-1)^(alpha-y)
    M = np.zeros((n + 1, n + 1))
    for y in range(n + 1):
        for al in range(y, n + 1):
            M[y, al] = comb(al, y) * (-1) ** (al - y)
    p = b
    for ax in range(k):
        p = np.moveaxis(np.tensordot(M, np.moveaxis(p, ax, 0), axes=(1, 0)), 0, ax)
    return np.clip(p, 0.0, None)


