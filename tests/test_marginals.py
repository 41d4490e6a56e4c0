"""CPU: the oracle's exact one- and two-mode marginals (binomial-moment
method, oracle/marginals.py) against brute-force sums of exact output
probabilities |perm|^2 / (prod y! prod x!) — the checker of the GPU marginals."""

import itertools
from math import factorial

import numpy as np
import pytest

import oracle
from conftest import haar_unitary
from oracle import marginals as omarg


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
        ex = omarg.marginal(inp, U, modes)
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
    for pair in [(0, 1), (2, 5), (3, 4)]:
        ex = omarg.marginal(inp, U, pair)
        em = np.zeros_like(ex)
        np.add.at(em, (samples[:, pair[0]], samples[:, pair[1]]), 1.0 / len(samples))
        assert 0.5 * np.abs(ex - em).sum() < 0.01, pair
