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


@pytest.fixture
def marginals_on_cpu(monkeypatch):
    """piquasso_gb300.marginals with its one device call (the binomial
    moments of many mode sets) replaced by the oracle's dynamic program."""
    from oracle import marginals as om

    from piquasso_gb300 import marginals

    def moments_sets(input_photons, U, mode_sets, max_device_bytes=0):
        return np.stack([om.binomial_moments(input_photons, U, list(s)) for s in mode_sets])

    monkeypatch.setattr(marginals, "binomial_moments_sets", moments_sets)
    return marginals


def test_marginal_host_logic(marginals_on_cpu):
    """The host side of the GPU marginals: the binomial transform, the
    postselected probabilities, the conditional marginal sampler and the TVD
    judge, against the oracle's marginals and brute-force sums."""
    from oracle import marginals as om

    mg = marginals_on_cpu
    d = 5
    U = haar_unitary(d, 12)
    inp = [1, 0, 2, 0, 1]
    n = sum(inp)
    for modes in ([0], [1, 3], [4, 2]):
        assert np.allclose(mg.marginal(inp, U, modes), om.marginal(inp, U, modes), atol=1e-13)
    # postselection: Pr(mode 1 has 1 photon and mode 3 has y) from the two-mode marginal
    joint = mg.marginal(inp, U, [1, 3])
    post = mg.get_marginal_fock_probabilities(inp, U, [1], [1], [3])
    assert set(post) == {(a,) for a in range(n)}
    for (a,), v in post.items():
        assert abs(v - joint[1, a]) < 1e-14
    # conditional sampler: its empirical two-mode distribution approaches the exact one
    S = mg.generate_marginal_samples(inp, U, [0, 2], 4000, seed=3)
    h = np.zeros((n + 1, n + 1))
    for a, b in S:
        h[a, b] += 1.0 / len(S)
    assert 0.5 * np.abs(h - mg.marginal(inp, U, [0, 2])).sum() < 0.04
    # the TVD check on samples drawn from the exact distribution of the pair
    rng = np.random.default_rng(0)
    pair = mg.marginal(inp, U, [0, 2])
    idx = rng.choice(pair.size, size=20000, p=pair.ravel() / pair.sum())
    full = np.zeros((20000, d), dtype=int)
    full[:, 0], full[:, 2] = np.unravel_index(idx, pair.shape)
    assert mg.tvd_two_mode(full, inp, U, [(0, 2)])[0] < 0.02
