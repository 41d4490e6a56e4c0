"""GPU tests of the autotuner: the planner applies a tuned entry to the
workloads in its ranges and only to them, results do not depend on the
tuning, and a short tuning run produces an entry that covers its workload."""

import ctypes

import numpy as np
import pytest

import oracle
from conftest import haar_unitary

pytestmark = pytest.mark.gpu


def _plan_config(plan):
    from piquasso_gb300 import _lib

    v = [ctypes.c_int64(0) for _ in range(3)]
    b = ctypes.c_int32(0)
    assert _lib.load().pqg_plan_config(plan._h, *[ctypes.byref(x) for x in v], ctypes.byref(b)) == 0
    return {"items_per_smsp": v[0].value, "p_max": v[1].value, "seed_steps": v[2].value, "blocks_per_sm": b.value}


@pytest.fixture
def table(engine):
    from piquasso_gb300 import autotune

    yield autotune
    autotune.apply_cache()  # the package's own table back


def test_planner_applies_matching_entry_only(engine, table):
    n = 18
    U = haar_unitary(2 * n, 5)[:n, :n].copy()
    o = np.ones(n, dtype=np.int64)
    steps = 2.0 ** (n - 1)
    table.install([{"form": "plain", "arith": "df", "nc": [n, n], "steps": [steps / 2, steps * 2],
                    "problems": [1, 2], "items_per_smsp": 4, "p_max": 64, "seed_steps": 128, "blocks_per_sm": 1}])
    with engine.PermanentPlan(U, o[None], o) as p:
        cfg = _plan_config(p)
        tuned = p.run()[0]
    assert cfg == {"items_per_smsp": 4, "p_max": 64, "seed_steps": 128, "blocks_per_sm": 1}
    # another arithmetic, and another size: the defaults
    with engine.PermanentPlan(U, o[None], o, mode="fp64") as p:
        assert _plan_config(p)["p_max"] != 64
    m = n - 2
    with engine.PermanentPlan(U[:m, :m].copy(), o[None, :m], o[:m]) as p:
        assert _plan_config(p)["p_max"] != 64
    table.install([])
    with engine.PermanentPlan(U, o[None], o) as p:
        default = p.run()[0]
    dd = oracle.permanent(U, o, o)
    tol = max(1e-10 * abs(dd), 1e-14 * oracle.perm_abs(U, o, o))
    assert abs(tuned - dd) <= tol and abs(default - dd) <= tol


def test_short_tuning_run_covers_its_workload(engine, table, tmp_path):
    n = 20
    U = haar_unitary(2 * n, 6)[:n, :n].copy()
    o = np.ones(n, dtype=np.int64)
    w = table.Workload("single_n20_df", U, o[None], o)
    cands = (("p_max", (0, 64, 256)), ("blocks_per_sm", (0, 1)))
    r = table.tune(w, reps=3, rounds=1, candidates=cands)
    assert r["tuned_ms"] <= r["default_ms"]
    e = r["entry"]
    assert e["form"] == "plain" and e["arith"] == "df" and e["nc"] == [n, n]
    assert e["steps"][0] <= 2.0 ** (n - 1) < e["steps"][1]
    assert e["problems"][0] <= 1 <= e["problems"][1]
    path = str(tmp_path / "cache.json")
    table.save([r], path, key="test|key")
    assert table.cached_entries("test|key", paths=[path])[0]["p_max"] == e["p_max"]
