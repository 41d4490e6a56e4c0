"""CPU tests of the autotuner's cache (piquasso_gb300.autotune): entries are
merged per workload range, keyed by GPU and library version, read user cache
first, and installed into the engine's table with the right codes.  No GPU:
the engine library is replaced by a recorder."""

import json

import numpy as np

from piquasso_gb300 import autotune


def _result(form="plain", arith="df", nc=28, steps=2.0 ** 27, probs=1, **knobs):
    s = dict(autotune.DEFAULT_SETTINGS, **knobs)
    return {"entry": {"form": form, "arith": arith, "nc": [nc, nc], "steps": [steps / 2, steps * 2],
                      "problems": [max(1, probs // 2), probs * 2], "workload": "w", **s}}


def test_save_merges_by_workload_range(tmp_path):
    path = str(tmp_path / "t.json")
    autotune.save([_result(p_max=128), _result(arith="c64", seed_steps=512)], path, key="GPU|v1")
    autotune.save([_result(p_max=256)], path, key="GPU|v1")  # same range: replaces
    autotune.save([_result(p_max=64)], path, key="OTHER|v1")
    data = json.load(open(path))
    assert data["format"] == autotune.FORMAT
    lst = data["entries"]["GPU|v1"]
    assert len(lst) == 2
    assert {(e["arith"], e["p_max"]) for e in lst} == {("df", 256), ("c64", 0)}
    assert autotune.cached_entries("OTHER|v1", paths=[path])[0]["p_max"] == 64
    assert autotune.cached_entries("NONE|v1", paths=[path]) == []


def test_user_cache_comes_before_the_shipped_one(tmp_path):
    user, shipped = str(tmp_path / "u.json"), str(tmp_path / "s.json")
    autotune.save([_result(p_max=32)], user, key="K")
    autotune.save([_result(p_max=512)], shipped, key="K")
    got = autotune.cached_entries("K", paths=[user, shipped])
    assert [e["p_max"] for e in got] == [32, 512]  # the engine takes the first match


def test_unreadable_or_foreign_caches_are_ignored(tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    old = tmp_path / "old.json"
    old.write_text(json.dumps({"format": 999, "entries": {"K": [{}]}}))
    assert autotune.cached_entries("K", paths=[str(bad), str(old), str(tmp_path / "missing.json")]) == []


class RecorderLib:
    def __init__(self):
        self.calls = []

    def pqg_tuning_clear(self):
        self.calls.append(("clear",))
        return 0

    def pqg_tuning_add(self, *args):
        self.calls.append(("add",) + args)
        return 0


def test_install_passes_codes_and_ranges():
    lib = RecorderLib()
    e = _result(form="laplace", arith="c64", nc=24, steps=1024.0, probs=2048, p_max=64, seed_steps=256,
                items_per_smsp=8, blocks_per_sm=2)["entry"]
    autotune.install([e], lib)
    assert lib.calls[0] == ("clear",)
    add = lib.calls[1]
    assert add[1:3] == (autotune.FORMS["laplace"], autotune.ARITHS["c64"])
    assert add[3:5] == (24, 24)
    assert add[5:7] == (512.0, 2048.0)
    assert add[7:9] == (1024, 4096)
    assert add[9:] == (8, 64, 256, 2)


def test_workload_stats_count_kept_columns_and_walk_problems():
    U = np.eye(6, dtype=complex)
    rows = np.array([[1, 1, 0, 0, 0, 0], [0, 0, 0, 0, 0, 0], [2, 0, 0, 0, 0, 0]])
    cols = np.array([[1, 0, 1, 0, 0, 0], [0, 0, 0, 0, 0, 0], [1, 1, 0, 0, 0, 0]])
    w = autotune.Workload("w", U, rows, cols)
    assert w.stats() == (2, 2)  # the empty problem needs no walk
    assert w.arith == "df" and autotune.Workload("w", U.astype(np.complex64), rows, cols).arith == "c64"
    assert autotune.Workload("w", U, rows, cols, mode="fp64").arith == "fp64"
