"""Concurrent engine calls from several host threads.

The engine's context lock serialises the device work, and the planner
configuration has its own lock, so that a thread plans its batch while
another thread's launch runs (capi.cu, Context::mu and Context::cfg_mu).
Reductions have a fixed order, so a permanent does not depend on which
thread computed it or on what ran beside it: concurrent results must equal
the sequential ones bit for bit, while a third thread edits the tuning table
with entries that match none of the workloads.
"""

import threading

import numpy as np
import pytest

from conftest import haar_unitary

pytestmark = pytest.mark.gpu


def _workloads():
    rng = np.random.default_rng(5)
    out = []
    for k in range(4):
        d, n = 24, 12
        U = haar_unitary(d, 20 + k)
        rows = np.stack([np.bincount(rng.integers(0, d, n), minlength=d) for _ in range(96)])
        cols = np.array([1] * n + [0] * (d - n))
        out.append((U if k % 2 else U.astype(np.complex64), rows, cols))
    return out


def test_concurrent_batches_match_sequential(engine):
    from piquasso_gb300 import _lib, autotune

    work = _workloads()
    want = [engine.permanent_batch(U, R, c) for U, R, c in work]
    got = [[None] * len(work) for _ in range(3)]
    errors = []

    def worker(t):
        try:
            for rep in range(3):
                for i in range(len(work)):
                    j = (i + t) % len(work)
                    U, R, c = work[j]
                    got[t][j] = engine.permanent_batch(U, R, c)
        except Exception as e:  # reported by the main thread
            errors.append(e)

    L = _lib.load()
    before = _lib.tuning_count()

    def tuner():
        try:
            for _ in range(200):
                # a Laplace double-float entry for 31 columns: no workload here matches it
                assert L.pqg_tuning_add(1, 1, 31, 31, 1.0, 2.0, 1, 1, 2, 64, 0, 0) == 0
                _lib.tuning_count()
        except Exception as e:
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(3)] + [threading.Thread(target=tuner)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    try:
        assert not errors, errors
        for t in range(3):
            for j in range(len(work)):
                assert np.array_equal(got[t][j], want[j]), (t, j)
        assert _lib.tuning_count() == before + 200
    finally:
        autotune.apply_cache(L)  # the shipped and user entries again, without the test's
