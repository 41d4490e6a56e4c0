"""Postselected exact boson sampling (piquasso_gb300.postselect).

* Against the reference: tests/golden/sampler_postselect_seeded.json holds
  the samples the reference's own sampling.py makes for seeded cases
  (lossless, multiphoton, a postselected count of zero, uniform loss,
  non-uniform loss through the dilation, partial distinguishability with and
  without loss), and its trial-limit message.  The CPU tests drive the host
  logic with the engine's Laplace call replaced by the oracle's
  double-double Laplace permanents; the GPU tests run the engine.
* Distribution: lossless postselected samples against the exact conditional
  distribution from brute-force permanents (oracle).
"""

import itertools
import json
import math
import os

import numpy as np
import pytest

import oracle
from conftest import haar_unitary

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "sampler_postselect_seeded.json")))


def _matrix(m):
    return (np.array(m["re"]) + 1j * np.array(m["im"])).astype(m["dtype"])


def _oracle_laplace_batch(U, rows, cols):
    """permanent_laplace_batch restated on the oracle: row b holds, for every
    column j with cols[b, j] > 0, the permanent with that column lowered."""
    rows, cols = np.atleast_2d(rows), np.atleast_2d(cols)
    out = np.zeros(cols.shape, dtype=np.complex128)
    for b, (r, c) in enumerate(zip(rows, cols)):
        if r.sum() == 0:
            continue  # the first photon: the pmf does not read the Laplace values
        out[b] = oracle.permanent_laplace_dd(U, r, c)[: cols.shape[1]]
    return out


@pytest.fixture
def ps_on_cpu(monkeypatch):
    from piquasso_gb300 import postselect

    monkeypatch.setattr(postselect, "permanent_laplace_batch", _oracle_laplace_batch)
    return postselect


def _run(sampling, case):
    U = _matrix(case["matrix"])
    return sampling.sample(np.array(case["input"]), case["shots"], U, case["seed"],
                           particle_overlap=case["overlap"], postselect=(case["modes"], case["photons"]))


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_reference_samples_on_cpu(ps_on_cpu, case):
    from piquasso_gb300 import sampling

    got = _run(sampling, case)
    assert [list(s) for s in got] == case["samples"]


def test_trial_limit_message(ps_on_cpu):
    from piquasso_gb300 import sampling

    t = GOLDEN["trial_limit"]
    with pytest.raises(ps_on_cpu.InvalidSimulation) as e:
        sampling.sample(np.array(t["input"]), 1, _matrix(t["matrix"]), 0,
                        postselect=(t["modes"], t["photons"], t["max_trials"]))
    assert str(e.value) == t["message"]


def test_lossless_overlap_does_not_fail(ps_on_cpu):
    """The reference raises here (a loss weight of about -1e-16 for a
    unitary, recorded in the golden file); the port clamps it at zero."""
    from piquasso_gb300 import sampling

    assert GOLDEN["lossless_overlap"]["raises"].startswith("ValueError")
    S = sampling.sample(np.array([1, 1, 1, 0, 0]), 30, haar_unitary(5, 11), 3, particle_overlap=0.5,
                        postselect=((0,), (1,)))
    assert len(S) == 30 and all(len(s) == 4 and sum(s) == 2 for s in S)


def test_invalid_postselection_arguments(ps_on_cpu):
    from piquasso_gb300 import sampling

    U = haar_unitary(4, 1)
    with pytest.raises(ValueError):
        sampling.sample(np.array([1, 1, 0, 0]), 2, U, 0, postselect=((0, 1), (1,)))
    with pytest.raises(ValueError):
        sampling.sample(np.array([1, 1, 0, 0]), 2, U, 0, postselect=((4,), (1,)))
    with pytest.raises(ValueError):
        sampling.sample(np.array([1, 1, 0, 0]), 2, U, 0, postselect=((0, 0), (1, 1)))


def _conditional(U, inp, modes, counts):
    """Exact distribution of the other modes given the postselected counts
    (brute force over every output pattern with the oracle's permanents)."""
    d, n = len(inp), int(sum(inp))
    keep = [m for m in range(d) if m not in modes]
    probs = {}
    for out in itertools.product(range(n + 1), repeat=d):
        if sum(out) != n or any(out[m] != c for m, c in zip(modes, counts)):
            continue
        a = complex(oracle.permanent(U, np.array(out), np.array(inp)))
        p = abs(a) ** 2 / (np.prod([math.factorial(x) for x in out]) * np.prod([math.factorial(x) for x in inp]))
        key = tuple(out[m] for m in keep)
        probs[key] = probs.get(key, 0.0) + p
    z = sum(probs.values())
    return {k: v / z for k, v in probs.items()}


def test_lossless_distribution(ps_on_cpu):
    from piquasso_gb300 import sampling

    U = haar_unitary(4, 21)
    inp = [1, 1, 1, 0]
    modes, counts = (1,), (1,)
    exact = _conditional(U, inp, modes, counts)
    S = sampling.sample(np.array(inp), 2500, U, 99, postselect=(modes, counts))
    emp = {}
    for s in S:
        emp[s] = emp.get(s, 0) + 1.0 / len(S)
    tvd = 0.5 * sum(abs(emp.get(k, 0.0) - exact.get(k, 0.0)) for k in set(emp) | set(exact))
    assert tvd < 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_reference_samples_on_gpu(case):
    from piquasso_gb300 import sampling

    got = _run(sampling, case)
    assert [list(s) for s in got] == case["samples"]


@pytest.mark.gpu
def test_trial_limit_on_gpu():
    from piquasso_gb300 import postselect, sampling

    t = GOLDEN["trial_limit"]
    with pytest.raises(postselect.InvalidSimulation) as e:
        sampling.sample(np.array(t["input"]), 1, _matrix(t["matrix"]), 0,
                        postselect=(t["modes"], t["photons"], t["max_trials"]))
    assert str(e.value) == t["message"]


@pytest.fixture
def batched_on_cpu(monkeypatch):
    from piquasso_gb300 import sampling
    from test_sampling_host_cpu import _numpy_step

    monkeypatch.setattr(sampling, "sampler_step_batch", _numpy_step)
    return sampling


def test_batched_rejection_distribution(batched_on_cpu):
    U = haar_unitary(4, 21)
    inp = [1, 1, 1, 0]
    modes, counts = (1,), (1,)
    exact = _conditional(U, inp, modes, counts)
    S = batched_on_cpu.sample(np.array(inp), 2500, U, 99, postselect=(modes, counts), batched=True)
    assert S.shape == (2500, 3) and np.all(S.sum(axis=1) == 2)
    emp = {}
    for s in map(tuple, S):
        emp[s] = emp.get(s, 0) + 1.0 / len(S)
    tvd = 0.5 * sum(abs(emp.get(k, 0.0) - exact.get(k, 0.0)) for k in set(emp) | set(exact))
    assert tvd < 0.05


def test_batched_rejection_lossy_trim_and_limits(batched_on_cpu):
    U = haar_unitary(5, 32) @ np.diag([0.9, 0.8, 0.95, 0.7, 0.85]) @ haar_unitary(5, 33)
    inp = np.array([1, 1, 1, 0, 0])
    S = batched_on_cpu.sample(inp, 200, U, 4, postselect=((2,), (1,)), batched=True)
    assert S.shape == (200, 5)  # postselected mode deleted from the 10 dilated modes, first 5 kept
    assert np.all(S[:, :4].sum(axis=1) <= 2)
    a = batched_on_cpu.sample(inp, 50, U, 6, postselect=((2,), (1,)), batched=True)
    b = batched_on_cpu.sample(inp, 50, U, 6, postselect=((2,), (1,)), batched=True)
    assert np.array_equal(a, b)
    from piquasso_gb300 import postselect

    with pytest.raises(postselect.InvalidSimulation):
        batched_on_cpu.sample(np.array([2, 0, 2, 0]), 3, haar_unitary(4, 16), 0, postselect=((0,), (5,), 4),
                              batched=True)
    assert batched_on_cpu.sample(inp, 0, haar_unitary(5, 2), 1, postselect=((0,), (1,)), batched=True).shape == (0, 4)


@pytest.mark.gpu
def test_batched_rejection_on_gpu():
    from piquasso_gb300 import sampling

    U = haar_unitary(4, 21)
    inp = [1, 1, 1, 0]
    exact = _conditional(U, inp, (1,), (1,))
    S = sampling.sample(np.array(inp), 4000, U, 99, postselect=((1,), (1,)), batched=True)
    assert S.shape == (4000, 3) and np.all(S.sum(axis=1) == 2)
    emp = {}
    for s in map(tuple, S):
        emp[s] = emp.get(s, 0) + 1.0 / len(S)
    assert 0.5 * sum(abs(emp.get(k, 0.0) - exact.get(k, 0.0)) for k in set(emp) | set(exact)) < 0.05
