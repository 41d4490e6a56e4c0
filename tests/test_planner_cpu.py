"""The host planner's invariants, on CPU: plan.cpp compiled with g++ beside a
small program (tests/planner/plan_dump.cpp) that prints a plan as JSON.

* outputs stay in the caller's order although problems are laid out longest
  item first (PqgProblem::index / out_of);
* items: consistent prefix sums; the complex64 plain walk's problems come in
  whole groups of four items (one per warp of a block); the lanes of a
  problem fill its items (whole warps);
* table lengths: P within the arithmetic's cap (256 for the FP32-pipe plain
  walks, which the 17..24-column complex64 kernel stages in shared memory;
  512 for FP64 and every Laplace walk);
* the double-float Laplace walk's domain (product over digits of
  C(m, m/2) <= 2^24) and the planner's input errors.
"""

import json
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "piquasso_gb300", "csrc")

C128, C64, DF = 0, 1, 2


@pytest.fixture(scope="module")
def planner(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("planner") / "plan_dump")
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", CSRC, os.path.join(HERE, "planner", "plan_dump.cpp"),
                    os.path.join(CSRC, "plan.cpp"), "-o", exe], check=True, capture_output=True)

    def run(prec, form, rows, cols):
        rows = np.atleast_2d(np.asarray(rows, dtype=int))
        cols = np.atleast_2d(np.asarray(cols, dtype=int))
        if cols.shape[0] == 1 and rows.shape[0] > 1:
            cols = np.repeat(cols, rows.shape[0], axis=0)
        lines = ["%d %d %d %d %d" % (prec, form, rows.shape[1], cols.shape[1], rows.shape[0])]
        for r, c in zip(rows, cols):
            lines.append(" ".join(map(str, r)) + " " + " ".join(map(str, c)))
        out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
        return json.loads(out.stdout)

    return run


def _check_layout(plan, batch):
    probs = plan["probs"]
    assert sorted(p["index"] for p in probs) == list(range(batch))
    # outputs in caller order
    n_out = {p["index"]: p["n_out"] for p in probs}
    acc = 0
    for b in range(batch):
        assert plan["out_of"][b] == acc
        acc += n_out[b]
    assert plan["total_outputs"] == acc
    for p in probs:
        assert p["out_index"] == plan["out_of"][p["index"]]
    # items: prefix sums in work order, whole groups, whole warps
    g = plan["item_group"]
    assert plan["total_items"] % g == 0
    for i, p in enumerate(probs):
        assert plan["item_begin"][i] == p["item_begin"]
        assert plan["item_begin"][i + 1] - plan["item_begin"][i] == p["n_items"]
        if p["kind"] != 0:
            assert p["n_items"] == 0
            continue
        assert p["n_items"] % g == 0 and p["item_begin"] % g == 0
        lanes = -(-p["Q"] // p["R"])
        assert p["n_items"] == -(-(-(-lanes // 32)) // g) * g
        assert p["P"] * p["Q"] == p["S"]
    assert plan["item_begin"][-1] == plan["total_items"]


@pytest.mark.parametrize("prec", [C128, C64, DF])
@pytest.mark.parametrize("form", [0, 1])
def test_random_batches(planner, prec, form):
    rng = np.random.default_rng(prec * 10 + form)
    d = 26
    R, C = [], []
    for b in range(60):
        n = int(rng.integers(0, 22)) if b % 11 else 0
        R.append(np.bincount(rng.integers(0, d, n), minlength=d))
        if form == 1 and n == 0:
            C.append(np.zeros(d, dtype=int))
        elif b % 2:
            c = np.zeros(d, dtype=int)
            c[rng.permutation(d)[:n]] = 1
            C.append(c)
        else:
            C.append(np.bincount(rng.integers(0, d, n), minlength=d))
    plan = planner(prec, form, R, C)
    assert "error" not in plan, plan
    _check_layout(plan, len(R))
    assert plan["item_group"] == (4 if (prec == C64 and form == 0) else 1)
    cap = 512 if (prec == C128 or form == 1) else 256
    for p in plan["probs"]:
        assert p["P"] <= cap


def test_longest_items_first(planner):
    """One large and many small problems: the large one is walked first
    although it comes last in the caller's order."""
    d = 24
    R = [np.eye(d, dtype=int)[i % d] for i in range(20)] + [np.ones(d, dtype=int)]
    C = [np.eye(d, dtype=int)[(3 * i) % d] for i in range(20)] + [np.ones(d, dtype=int)]
    plan = planner(C64, 0, R, C)
    _check_layout(plan, len(R))
    assert plan["probs"][0]["index"] == 20


def test_whole_warps_fill_items(planner):
    """A problem of a few thousand outer positions fills whole warps rather
    than leaving a mostly idle last item."""
    d = 24
    rows = np.ones(d, dtype=int)
    plan = planner(C128, 0, [rows] * 3, [np.ones(d, dtype=int)])
    _check_layout(plan, 3)
    for p in plan["probs"]:
        lanes = -(-p["Q"] // p["R"])
        assert lanes > 32 * (p["n_items"] - 1) + 16  # the last item is more than half full


def test_double_float_laplace_domain(planner):
    d = 8
    cols = np.ones(d, dtype=int) * 2
    ok = planner(DF, 1, [[2] * 8], [cols])
    assert ok["df_ok"] == 1
    # one row with 16 photons: C(15, 7) = 6435; two such rows exceed 2^24 together
    big = planner(DF, 1, [[16, 16, 0, 0, 0, 0, 0, 0]], [[4] * 8])
    assert big["df_ok"] == 0


def test_input_errors(planner):
    assert planner(C128, 0, [[1, -1, 2]], [[1, 1, 0]])["error"] == 2
    assert planner(C128, 0, [[1, 1, 1]], [[1, 1, 0]])["error"] == 1  # sum mismatch
    many = planner(C128, 0, [[1] * 33], [[1] * 33])
    assert many["error"] == 3  # more than 32 distinct columns


@pytest.mark.parametrize("prec,form", [(C64, 0), (DF, 1), (C128, 1)])
def test_threaded_planning_is_deterministic(planner, monkeypatch, prec, form):
    """From 2048 problems on, add_batch and finish plan on several host
    threads; the plan (problem records, arena bytes, layout) is the same as
    on one thread."""
    rng = np.random.default_rng(40 + prec + form)
    d, n = 40, 12
    R, C = [], []
    for b in range(2600):
        R.append(np.bincount(rng.integers(0, d, n), minlength=d))
        c = np.zeros(d, dtype=int)
        c[rng.permutation(d)[:n]] = 1
        C.append(c if b % 3 else np.bincount(rng.integers(0, d, n), minlength=d))
    monkeypatch.setenv("PQG_HOST_THREADS", "1")
    one = planner(prec, form, R, C)
    monkeypatch.setenv("PQG_HOST_THREADS", "4")
    four = planner(prec, form, R, C)
    assert "error" not in one, one
    _check_layout(four, len(R))
    assert one == four


@pytest.mark.parametrize("prec,form", [(C64, 0), (DF, 1)])
def test_pooled_buffers_give_the_same_plan(planner, monkeypatch, prec, form):
    """A planner reuses the buffers of the last planner destroyed on its
    thread; a plan made after another (different) plan on dirty buffers is
    byte for byte the plan of a fresh process."""
    rng = np.random.default_rng(50 + prec + form)
    d, n = 30, 10
    R = [np.bincount(rng.integers(0, d, n), minlength=d) for _ in range(300)]
    C = [np.bincount(rng.integers(0, d, n), minlength=d) for _ in range(300)]
    fresh = planner(prec, form, R, C)
    monkeypatch.setenv("PLAN_DUMP_WARM", "1")
    warm = planner(prec, form, R, C)
    assert "error" not in fresh, fresh
    assert fresh == warm


def test_threaded_planning_reports_the_first_bad_problem(planner, monkeypatch):
    d = 6
    R = [[1, 1, 0, 0, 0, 0]] * 3000
    C = [[1, 1, 0, 0, 0, 0]] * 3000
    R[2100] = [1, 1, 1, 0, 0, 0]  # sum mismatch
    R[2900] = [1, -1, 2, 0, 0, 0]  # negative multiplicity, later
    monkeypatch.setenv("PQG_HOST_THREADS", "4")
    bad = planner(C128, 0, R, C)
    assert bad["error"] == 1 and bad["problem"] == 2100


def test_code_pair_tables(planner):
    """complex64 Laplace plans whose walk problems all have unit columns (up
    to 24 of them) store their prefix tables as code pairs for the two-code
    walk: each problem's table holds an even number of codes (an odd P gets a
    pad code), so every table starts at an even slot and the float4 pair
    rows stay aligned; any other plan keeps P codes per problem."""
    rng = np.random.default_rng(7)
    d, n = 30, 12
    inp = np.array([1] * n + [0] * (d - n))
    rows = np.stack([np.bincount(rng.integers(0, d, n - 1), minlength=d) for _ in range(40)])
    plan = planner(C64, 1, rows, inp)
    assert plan["pairs"] == 1
    walk = [p for p in plan["probs"] if p["kind"] == 0]
    assert any(p["P"] % 2 for p in walk)  # odd tables occur and get padded
    total = 0
    for p in sorted(walk, key=lambda p: p["delta_begin"]):
        assert p["delta_begin"] == total and p["delta_begin"] % 2 == 0
        total += (p["P"] + p["P"] % 2) * p["nc"]
    assert plan["total_delta"] == total
    # a repeated column, more than 24 columns, another arithmetic or the plain form: no pairs
    inp2 = inp.copy()
    inp2[0] = 2
    rows2 = rows.copy()
    rows2[:, 0] += 1
    assert planner(C64, 1, rows2, inp2)["pairs"] == 0
    wide = np.array([1] * 26 + [0] * 4)
    rows3 = np.stack([np.bincount(rng.integers(0, d, 25), minlength=d) for _ in range(4)])
    assert planner(C64, 1, rows3, wide)["pairs"] == 0
    assert planner(C128, 1, rows, inp)["pairs"] == 0
    assert planner(C64, 0, np.stack([np.bincount(rng.integers(0, d, n), minlength=d) for _ in range(4)]),
                   inp)["pairs"] == 0
