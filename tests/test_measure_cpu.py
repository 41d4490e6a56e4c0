"""ParticleNumberMeasurement's dispatch (piquasso_gb300.sampling.measure) on
CPU: the reference's rule for direct marginal sampling, the active-mode
numbering after a postselection, and both branches.  The marginal branch
runs the real host code over the oracle's exact marginals, and the full
branch runs the postselected sampler with the oracle's Laplace permanents in
place of the engine."""

import numpy as np
import pytest

from conftest import haar_unitary
from oracle import marginals as omarg
from test_postselect import _oracle_laplace_batch


def test_cheaper_rule():
    from piquasso_gb300.sampling import is_direct_marginal_sampling_cheaper as cheaper

    # coefficient counts sum_{m<=n} C(m+k-1, k-1)^2: (3, 16) 93993; (3, 20) 256795;
    # (4, 16) 2904093; (5, 12) 7109128
    assert not cheaper(k=4, d=4, n=2, shots=10**6)  # every mode
    assert cheaper(k=3, d=10, n=16, shots=1)
    assert cheaper(k=3, d=10, n=20, shots=1000) and not cheaper(k=3, d=10, n=20, shots=999)
    assert cheaper(k=4, d=10, n=16, shots=10_000) and not cheaper(k=4, d=10, n=16, shots=9_999)
    assert not cheaper(k=5, d=10, n=12, shots=10**9)


def test_map_to_original_modes():
    from piquasso_gb300.sampling import map_to_original_modes

    assert map_to_original_modes((0, 1, 2), (1,)) == (0, 2, 3)
    assert map_to_original_modes((0, 1), (0, 2)) == (1, 3)
    assert map_to_original_modes((1, 0), ()) == (1, 0)


@pytest.fixture
def on_cpu(monkeypatch):
    from piquasso_gb300 import marginals, postselect

    calls = {"marginal": 0}

    def marginal(inp, U, modes):
        calls["marginal"] += 1
        return omarg.marginal(inp, U, list(modes))

    monkeypatch.setattr(marginals, "marginal", marginal)
    monkeypatch.setattr(postselect, "permanent_laplace_batch", _oracle_laplace_batch)
    return calls


def test_marginal_branch_with_postselection(on_cpu):
    from piquasso_gb300 import sampling

    U = haar_unitary(5, 31)
    inp = [1, 1, 1, 0, 0]
    shots = 4000
    counts = sampling.measure(np.array(inp), shots, U, 8, modes=(1,), postselect=((0,), (1,)))
    assert on_cpu["marginal"] == 1  # the direct marginal sampler ran
    assert sum(counts.values()) == shots and all(len(k) == 1 for k in counts)
    # active mode 1 is original mode 2: Pr(Y_2 = y | Y_0 = 1)
    joint = omarg.marginal(inp, U, [0, 2])[1]
    exact = joint / joint.sum()
    emp = np.zeros(len(exact))
    for (y,), c in counts.items():
        emp[y] += c / shots
    assert 0.5 * np.abs(emp - exact).sum() < 0.04


def test_full_branch_projects_postselected_samples(on_cpu):
    from piquasso_gb300 import postselect, sampling

    U = haar_unitary(5, 32) @ np.diag([0.9, 0.8, 0.95, 0.7, 0.85]) @ haar_unitary(5, 33)
    inp = np.array([1, 1, 1, 0, 0])
    ps = ((2,), (1,))
    counts = sampling.measure(inp, 40, U, 4, modes=(0, 3), postselect=ps)
    assert on_cpu["marginal"] == 0  # non-uniform loss: never the marginal branch
    full = postselect.generate_lossy_samples(inp, 40, U, 4, ps)
    expect = {}
    for s in full:
        key = (s[0], s[3])
        expect[key] = expect.get(key, 0) + 1
    assert counts == expect


def test_every_mode_measured(on_cpu):
    from piquasso_gb300 import sampling

    U = haar_unitary(4, 34)
    counts = sampling.measure(np.array([1, 1, 0, 1]), 30, U, 2, postselect=((3,), (0,)))
    assert on_cpu["marginal"] == 0
    assert sum(counts.values()) == 30
    assert all(len(k) == 3 and sum(k) == 3 for k in counts)
