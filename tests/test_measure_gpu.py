"""ParticleNumberMeasurement's dispatch (sampling.measure) on the GPU engine:
the direct marginal branch after a postselection against the oracle's exact
conditional marginal, and the full branch's projection."""

import numpy as np
import pytest

from conftest import haar_unitary
from oracle import marginals as omarg

pytestmark = pytest.mark.gpu


def test_marginal_branch_on_gpu(engine):
    from piquasso_gb300 import sampling

    U = haar_unitary(5, 31)
    inp = [1, 1, 1, 0, 0]
    shots = 6000
    counts = sampling.measure(np.array(inp), shots, U, 8, modes=(1,), postselect=((0,), (1,)))
    assert sum(counts.values()) == shots
    joint = omarg.marginal(inp, U, [0, 2])[1]  # active mode 1 is original mode 2
    exact = joint / joint.sum()
    emp = np.zeros(len(exact))
    for (y,), c in counts.items():
        emp[y] += c / shots
    assert 0.5 * np.abs(emp - exact).sum() < 0.04


def test_full_branch_on_gpu(engine):
    from piquasso_gb300 import sampling

    U = haar_unitary(5, 32) @ np.diag([0.9, 0.8, 0.95, 0.7, 0.85]) @ haar_unitary(5, 33)
    counts = sampling.measure(np.array([1, 1, 1, 0, 0]), 40, U, 4, modes=(0, 3), postselect=((2,), (1,)))
    assert sum(counts.values()) == 40 and all(len(k) == 2 and sum(k) <= 2 for k in counts)
    full = sampling.measure(np.array([1, 1, 0, 1]), 30, haar_unitary(4, 34), 2, batched=True)
    assert sum(full.values()) == 30 and all(len(k) == 4 and sum(k) == 3 for k in full)
