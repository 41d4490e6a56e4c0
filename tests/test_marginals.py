"""CPU: exact one- and two-mode marginals (binomial-moment method) against
brute-force sums of exact output probabilities |perm|^2 / (prod y! prod x!)."""

import itertools
from math import factorial

import numpy as np
import pytest

import oracle
from conftest import haar_unitary
from piquasso_gb300 import marginals


def _all_patterns(n, d):
    for c in itertools.combinations_with_replacement(range(d), n):
        yield np.bincount(c, minlength=d)


def _brute(inp, U, modes):
    n = int(sum(inp))
    out = np.zeros((n + 1,) * len(modes))
    norm = np.prod([factorial(x) for x in inp])
    for y in _all_patterns(n, len(inp)):
        p = abs(oracle.permanent(U, y, inp)) ** 2 / (norm * np.prod([factorial(v) for v in y]))
        out[tuple(y[m] for m in modes)] += p
    return out


@pytest.mark.parametrize("inp", [[1, 1, 1, 0, 0], [2, 1, 0, 1, 0], [1, 0, 3, 0, 0]])
def test_marginals_match_brute_force(inp):
    U = haar_unitary(len(inp), 11)
    for modes in ((0,), (3,), (0, 1), (2, 4), (4, 1)):
        ex = marginals.marginal(inp, U, modes)
        bf = _brute(inp, U, modes)
        assert np.allclose(ex, bf, atol=1e-12), (modes, ex, bf)
        assert abs(ex.sum() - 1) < 1e-12


def test_tvd_of_exact_distribution_is_small():
    inp = [1, 1, 1, 0, 0, 0]
    U = haar_unitary(6, 5)
    rng = np.random.default_rng(0)
    pats = list(_all_patterns(3, 6))
    probs = np.array([abs(oracle.permanent(U, y, inp)) ** 2 / np.prod([factorial(v) for v in y]) for y in pats])
    probs /= probs.sum()
    idx = rng.choice(len(pats), size=200000, p=probs)
    samples = np.array(pats)[idx]
    tv = marginals.tvd_two_mode(samples, inp, U, [(0, 1), (2, 5), (3, 4)])
    assert np.all(tv < 0.01), tv
