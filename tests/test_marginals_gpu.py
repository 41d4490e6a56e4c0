"""GPU: exact marginals from the engine's binomial-moment dynamic program
(pqg_binomial_moments_c128) against the CPU restatement (oracle/marginals.py,
one and two modes) and against brute-force sums of exact output
probabilities |perm|^2 / (prod y! prod x!) for three and four modes; several
mode sets per call; the reference's postselected form; the marginal sampler.

Tolerance: 1e-12 absolute on probabilities (FP64 sums of at most a few
thousand terms of magnitude <= 1); sampler: TVD below 0.01 at 100k samples.
"""

import itertools
from math import factorial

import numpy as np
import pytest

import oracle
from conftest import haar_unitary
from oracle import marginals as omarg

pytestmark = pytest.mark.gpu


def _patterns(n, d):
    for c in itertools.combinations_with_replacement(range(d), n):
        yield np.bincount(c, minlength=d)


def _brute(inp, U, modes):
    n = int(sum(inp))
    out = np.zeros((n + 1,) * len(modes))
    norm = np.prod([factorial(x) for x in inp])
    for y in _patterns(n, len(inp)):
        p = abs(oracle.permanent(U, y, inp)) ** 2 / (norm * np.prod([factorial(v) for v in y]))
        out[tuple(y[m] for m in modes)] += p
    return out


@pytest.mark.parametrize("inp", [[1, 1, 1, 0, 0], [2, 1, 0, 1, 0], [1, 0, 3, 0, 0], [0, 0, 0, 0, 0]])
def test_one_and_two_modes_match_restatement(engine, inp):
    from piquasso_gb300 import marginals

    U = haar_unitary(len(inp), 11)
    for modes in ((0,), (3,), (0, 1), (2, 4), (4, 1)):
        g = marginals.marginal(inp, U, modes)
        c = omarg.marginal(inp, U, modes)
        assert g.shape == c.shape
        assert np.max(np.abs(g - c)) < 1e-12, modes


@pytest.mark.parametrize("modes", [(0, 2, 4), (5, 1, 3, 0), (1, 2, 3, 4)])
def test_three_and_four_modes_match_brute_force(engine, modes):
    from piquasso_gb300 import marginals

    inp = [1, 2, 0, 1, 0, 0]
    U = haar_unitary(6, 2)
    g = marginals.marginal(inp, U, modes)
    b = _brute(inp, U, modes)
    assert np.max(np.abs(g - b)) < 1e-12
    assert abs(g.sum() - 1.0) < 1e-12


def test_many_sets_in_one_call(engine):
    from piquasso_gb300 import marginals

    inp = [1, 1, 0, 1, 1, 0, 0, 0]
    U = haar_unitary(8, 4)
    sets = [(0, 1), (2, 7), (5, 6), (3, 3), (7, 0)]
    many = marginals.marginals(inp, U, sets)
    for i, s in enumerate(sets):
        assert np.array_equal(many[i], marginals.marginal(inp, U, s))


def test_postselected_probabilities(engine):
    from piquasso_gb300 import marginals

    inp = [1, 1, 1, 0, 0]
    U = haar_unitary(5, 9)
    got = marginals.get_marginal_fock_probabilities(inp, U, (3,), (1,), (0, 4))
    b = _brute(inp, U, (3, 0, 4))
    assert set(got) == {(a, c) for a in range(3) for c in range(3) if a + c <= 2}
    for (a, c), p in got.items():
        assert abs(p - b[1, a, c]) < 1e-12


def test_larger_dynamic_program(engine):
    """n = 12 photons, four modes: nonnegative, normalised, consistent with
    its own two-mode marginals."""
    from piquasso_gb300 import marginals

    inp = [1] * 12 + [0] * 12
    U = haar_unitary(24, 31)
    p4 = marginals.marginal(inp, U, (0, 5, 11, 20))
    assert p4.min() > -1e-12 and abs(p4.sum() - 1.0) < 1e-10
    p2 = marginals.marginal(inp, U, (0, 5))
    assert np.max(np.abs(p4.sum(axis=(2, 3)) - p2)) < 1e-12


def test_marginal_sampler(engine):
    from piquasso_gb300 import marginals

    inp = [1, 1, 1, 1, 0, 0]
    U = haar_unitary(6, 14)
    S = np.array(marginals.generate_marginal_samples(inp, U, (1, 4), 100000, 3))
    ex = marginals.marginal(inp, U, (1, 4))
    em = np.zeros_like(ex)
    np.add.at(em, (S[:, 0], S[:, 1]), 1.0 / len(S))
    assert 0.5 * np.abs(ex - em).sum() < 0.01
    # postselected on mode 0 holding one photon: conditional distribution
    S2 = np.array(marginals.generate_marginal_samples(inp, U, (2,), 50000, 4, (0,), (1,)))
    joint = marginals.marginal(inp, U, (0, 2))[1]
    cond = joint / joint.sum()
    em2 = np.bincount(S2[:, 0], minlength=len(cond))[: len(cond)] / len(S2)
    assert 0.5 * np.abs(cond - em2).sum() < 0.01
