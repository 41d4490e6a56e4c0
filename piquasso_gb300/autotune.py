"""Autotuner of the permanent engine's work split.

The reference splits every permanent into 4 x hardware_concurrency contiguous
Gray-code segments, one per OpenMP thread (src/permanent.cpp:144-155).  This
engine's planner has four knobs instead (include/pqperm_gb300.h):

* ``p_max``: the longest inner walk, i.e. prefix-table length;
* ``seed_steps``: Gray-code steps per lane that amortise one seed;
* ``items_per_smsp``: warps of work per SM sub-partition the split aims for;
* ``blocks_per_sm``: resident walk blocks per SM.

:func:`tune` measures candidates of each knob in turn on one workload
(coordinate descent, every candidate timed with CUDA events over a few
executions of one graph-captured plan) and keeps the fastest.  The winners
go into a JSON cache keyed by GPU name and library version.  On load, the
package fills the engine's tuning table from that cache, so every later call
whose workload falls in a tuned entry's ranges (form, arithmetic, largest
column count, total Gray-code steps, number of problems) is planned with the
tuned knobs; other workloads keep the defaults.

The package ships a cache measured on a GB300 (``data/tuning.json``); a
user cache (``PQG_TUNING_CACHE``, default ``~/.cache/piquasso_gb300/
tuning.json``) overrides its entries.  ``python -m piquasso_gb300.autotune``
tunes the standard workloads (the benchmarked shapes) and writes the user
cache.
"""

import argparse
import datetime
import json
import os
import statistics
import time

import numpy as np

from . import _lib

SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "tuning.json")
FORMAT = 1
FORMS = {"plain": 0, "laplace": 1}
ARITHS = {"fp64": 0, "df": 1, "c64": 2}
# candidate values of each knob, in the order coordinate descent visits them
# (0 keeps the engine's default)
CANDIDATES = (
    ("p_max", (0, 32, 64, 128, 256, 512, 1024)),
    ("seed_steps", (0, 64, 128, 256, 512, 1024, 2048, 4096)),
    ("items_per_smsp", (0, 2, 4, 8, 16, 32, 64)),
    ("blocks_per_sm", (0, 1, 2, 3, 4)),
)
DEFAULT_SETTINGS = {"p_max": 0, "seed_steps": 0, "items_per_smsp": 0, "blocks_per_sm": 0}


def user_cache_path():
    return os.environ.get("PQG_TUNING_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "piquasso_gb300", "tuning.json")


def cache_key(lib=None):
    """'<GPU name>|<library version>': tuned settings apply to that pair only."""
    lib = lib or _lib.load()
    name, _ = _lib.device_info()
    return "%s|%s" % (name, lib.pqg_version().decode())


def _read(path):
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return {}
    return data.get("entries", {}) if data.get("format") == FORMAT else {}


def cached_entries(key=None, paths=None):
    """The tuned entries for `key` (default: this GPU and library), user cache
    first, then the shipped one."""
    key = key or cache_key()
    out = []
    for p in paths or (user_cache_path(), SHIPPED):
        out.extend(_read(p).get(key, []))
    return out


def install(entries, lib=None):
    """Replaces the engine's tuning table with `entries` (dicts as the cache
    stores them)."""
    lib = lib or _lib.load()
    lib.pqg_tuning_clear()
    for e in entries:
        st = lib.pqg_tuning_add(FORMS[e["form"]], ARITHS[e["arith"]], int(e["nc"][0]), int(e["nc"][1]),
                                float(e["steps"][0]), float(e["steps"][1]), int(e["problems"][0]),
                                int(e["problems"][1]), int(e["items_per_smsp"]), int(e["p_max"]),
                                int(e["seed_steps"]), int(e["blocks_per_sm"]))
        if st:
            raise ValueError("tuning entry %r: %s" % (e, _lib.last_error()))


def apply_cache(lib=None):
    """Loads this GPU's tuned entries into the engine (called on package load)."""
    lib = lib or _lib.load()
    install(cached_entries(cache_key(lib)), lib)


def save(results, path=None, key=None):
    """Merges tuning results (from :func:`tune`) into the cache at `path`
    (default: the user cache): an entry with the same form, arithmetic and
    ranges is replaced."""
    path = path or user_cache_path()
    key = key or cache_key()
    try:
        with open(path) as f:
            data = json.load(f)
        if data.get("format") != FORMAT:
            data = {}
    except (OSError, ValueError):
        data = {}
    data = {"format": FORMAT, "entries": data.get("entries", {})}
    lst = data["entries"].setdefault(key, [])
    for r in results:
        e = r["entry"]
        same = lambda x: all(x[k] == e[k] for k in ("form", "arith", "nc", "steps", "problems"))  # noqa: E731
        lst[:] = [x for x in lst if not same(x)] + [e]
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return path


class Workload:
    """A batch of permanents (or Laplace permanents) of one matrix, run as a
    graph-captured plan: ``rows`` (batch, n_rows), ``cols`` (batch, n_cols)
    or (n_cols,)."""

    def __init__(self, name, matrix, rows, cols, form="plain", mode="auto"):
        self.name = name
        self.matrix = np.asarray(matrix)
        self.rows = np.atleast_2d(np.asarray(rows)).astype(np.int64)
        c = np.asarray(cols).astype(np.int64)
        self.cols = np.broadcast_to(c, (self.rows.shape[0], c.shape[-1])) if c.ndim == 1 else c
        self.form = form
        self.mode = mode

    @property
    def arith(self):
        if self.matrix.dtype == np.complex64:
            return "c64"
        return "fp64" if self.mode == "fp64" else "df"

    def stats(self):
        """(largest column count, walk problems) after the reduction: columns
        of nonzero multiplicity; problems with photons on both sides."""
        rs, cs = self.rows.sum(1), self.cols.sum(1)
        walk = (rs > 0) & (cs > 0)
        nc = np.count_nonzero(self.cols, axis=1)
        return int(nc[walk].max()) if walk.any() else 0, int(walk.sum())

    def plan(self):
        from .plan import PermanentPlan

        return PermanentPlan(self.matrix, self.rows, self.cols, form=self.form, mode=self.mode)


def _set_knobs(s):
    _lib.set_tuning(s["items_per_smsp"], s["p_max"], s["seed_steps"])
    _lib.set_blocks_per_sm(s["blocks_per_sm"])


def time_workload(w, settings, reps=5):
    """Median device time (ms) of `reps` graph executions of the workload's
    plan, planned with `settings` (after one untimed execution), and the
    plan's Gray-code steps."""
    _set_knobs(settings)
    p = w.plan()
    try:
        p.launch()
        p.synchronize()
        ms = []
        for _ in range(reps):
            p.launch()
            ms.append(p.synchronize())
        steps = p.info()["steps"]
    finally:
        p.close()
    return statistics.median(ms), steps


def tune(w, reps=5, rounds=2, min_gain=0.01, candidates=CANDIDATES, log=None):
    """Coordinate descent over the knobs for workload `w`: each knob's
    candidates timed with the others fixed, a change kept when it is at least
    `min_gain` faster, until a round changes nothing.  The engine's tuning
    table is emptied while timing (so "default" is the engine's default) and
    restored after.  Returns a dict with the default and tuned times, the
    settings and the cache entry."""
    lib = _lib.load()
    saved = _lib.get_tuning()
    try:
        lib.pqg_tuning_clear()
        best = dict(DEFAULT_SETTINGS)
        base_ms, steps = time_workload(w, best, reps)
        best_ms, trials = base_ms, 1
        for _ in range(rounds):
            changed = False
            for knob, values in candidates:
                for v in values:
                    if v == best[knob]:
                        continue
                    s = dict(best, **{knob: v})
                    ms, _ = time_workload(w, s, reps)
                    trials += 1
                    if ms < best_ms * (1.0 - min_gain):
                        best, best_ms, changed = s, ms, True
                if log:
                    log("%s: %s -> %s (%.3f ms)" % (w.name, knob, best[knob], best_ms))
            if not changed:
                break
        # the winner against the default once more, back to back
        d_ms, _ = time_workload(w, DEFAULT_SETTINGS, reps)
        t_ms, _ = time_workload(w, best, reps)
        if t_ms >= d_ms:
            best, t_ms = dict(DEFAULT_SETTINGS), d_ms
    finally:
        _lib.set_tuning(saved["items_per_smsp"], 0 if saved["p_max"] == 2048 else saved["p_max"],
                        saved["seed_steps"])
        _lib.set_blocks_per_sm(0)
        apply_cache(lib)
    nc, probs = w.stats()
    entry = {"form": w.form, "arith": w.arith, "nc": [nc, nc], "steps": [steps / 2.0, steps * 2.0],
             "problems": [max(1, probs // 2), probs * 2], "workload": w.name,
             "default_ms": d_ms, "tuned_ms": t_ms,
             "when": datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%dT%H:%M:%SZ"), **best}
    return {"workload": w.name, "default_ms": d_ms, "tuned_ms": t_ms, "speedup": d_ms / t_ms,
            "settings": best, "trials": trials, "search_default_ms": base_ms, "entry": entry}


def standard_workloads():
    """The benchmarked shapes: the n = 24 and 28 single permanents (leading
    block of Haar(2n) seed 0) in the double-float, FP64 (n = 24) and complex64
    walks; the 4096-pattern batch of 20 photons in 40 modes (Haar(40) seed 1);
    a Metropolis block of 8192 complex64 target permanents (24 photons in 48
    modes, occupations <= 4, Haar(48) seed 3); the exact sampler's last
    photon step at n = 24, d = 48 (2048 complex64 Laplace problems)."""
    from . import workloads

    out = []
    for n in (24, 28):
        U = workloads.haar_unitary(2 * n, 0)[:n, :n].copy()
        o = np.ones(n, dtype=np.int64)
        out.append(Workload("single_n%d_df" % n, U, o[None], o, mode="auto"))
        out.append(Workload("single_n%d_c64" % n, U.astype(np.complex64), o[None], o))
    U = workloads.haar_unitary(48, 0)[:24, :24].copy()
    o = np.ones(24, dtype=np.int64)
    out.append(Workload("single_n24_fp64", U, o[None], o, mode="fp64"))
    U = workloads.haar_unitary(40, 1)
    inp = np.array([1] * 20 + [0] * 20)
    out.append(Workload("batch_4096_d40_n20", U, workloads.capped_compositions(20, 40, 4, 4096, seed=1), inp))
    rng = np.random.default_rng(7)
    d, n = 48, 24
    U = workloads.haar_unitary(d, 3)
    inp = np.array([1] * n + [0] * (d - n))
    R = []
    while len(R) < 8192:
        r = np.bincount(rng.integers(0, d, n), minlength=d)
        if r.max() <= 4:
            R.append(r)
    out.append(Workload("target_8192_n24_d48", U.astype(np.complex64), np.stack(R), inp))
    L = []
    while len(L) < 2048:
        r = np.bincount(rng.integers(0, d, n - 1), minlength=d)
        if r.max() <= 4:
            L.append(r)
    out.append(Workload("sampler_last_step_2048_n24_d48", U.astype(np.complex64), np.stack(L), inp,
                        form="laplace"))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description="Tune the permanent engine's work split on this GPU.")
    ap.add_argument("--out", default=None, help="cache file to write (default: the user cache)")
    ap.add_argument("--only", default=None, help="comma-separated workload names")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--rounds", type=int, default=2)
    a = ap.parse_args(argv)
    ws = standard_workloads()
    if a.only:
        keep = set(a.only.split(","))
        ws = [w for w in ws if w.name in keep]
    results = []
    for w in ws:
        t0 = time.perf_counter()
        r = tune(w, reps=a.reps, rounds=a.rounds, log=print)
        r["tune_s"] = time.perf_counter() - t0
        print(json.dumps({k: v for k, v in r.items() if k != "entry"}), flush=True)
        results.append(r)
    print("wrote", save(results, a.out))


if __name__ == "__main__":
    main()
