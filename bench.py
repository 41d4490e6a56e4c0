"""Benchmark: permanents per second at n=28 (complex128) on one GB300.

Workload: the leading 28x28 block of a seeded 56x56 Haar-random unitary
(QR of a complex Gaussian with the phase fix, seed 0), all row and column
multiplicities 1; one permanent per step, spread over every SM.  This is the
single-large-permanent configuration at the size the headline metric names.

Prints ONE JSON line (rank 0):
  value      permanents/s with the input resident on the device: device time
             of the whole pipeline (queue reset, walk, reductions) per step,
             CUDA events on the engine's stream, L2 flushed between steps;
  e2e        the same metric through the public API permanent(matrix, rows,
             cols) with host buffers: planning, host->device plan copy,
             kernels and the device->host result copy inside the timed region;
  roofline   the walk kernel against the measured FP64 FMA peak (algorithmic
             flops 2^(n-1)*(10n+4) per permanent / walk-kernel event time);
  cpu_baseline  the reference's CPU method (oracle port, all host threads)
             on the same input.
``--impl reference`` times that CPU method alone, on the same workload.
Multi-GPU (torchrun): independent replicas, one per rank; value = sum.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def haar_unitary(d, seed):
    rng = np.random.default_rng(seed)
    Z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    Q, R = np.linalg.qr(Z)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


# DRAM traffic of one n=28 double-float walk launch (bytes, read + write),
# recorded from an ncu capture of the headline workload on a GB300
TRAFFIC_N28_DF = 180992
TRAFFIC_N28_DF_DATE = "2026-12-04"


def hbm_gbs():
    """Measured HBM copy bandwidth of the GB300s (GB/s), or None."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return None


def flops_all_ones(n):
    return 2.0 ** (n - 1) * (10 * n + 4)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, interval_ms=25):
        self.gpu = gpu_index
        self.interval_ms = interval_ms
        self.proc = None
        self.path = None
        self.mark = 0

    def _lines(self):
        try:
            with open(self.path) as f:
                return sum(1 for line in f if line.count(",") >= 8)
        except OSError:
            return 0

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        return self

    def start_region(self):
        """Marks the start of the timed region: the samples taken from here on
        are the region's.  Entered before the warm-up, so that nvidia-smi's
        start-up does not fall into a short region."""
        t0 = time.perf_counter()
        while self.proc is not None and self._lines() == 0 and time.perf_counter() - t0 < 5.0 and \
                self.proc.poll() is None:
            time.sleep(0.01)
        self.mark = self._lines() if self.proc is not None else 0

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = [line for line in open(self.path) if line.count(",") >= 8]
        # the samples taken during the region (the last one before it if the
        # region was shorter than one interval)
        rows = rows[self.mark:] or rows[max(0, self.mark - 1):self.mark]
        for line in rows:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo", init_method="env://")
        pg = dist
    return world, rank, local, pg


def allreduce_max_sum(pg, vals_max, vals_sum):
    if pg is None:
        return vals_max, vals_sum
    import torch

    t = torch.tensor(vals_max, dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    s = torch.tensor(vals_sum, dtype=torch.float64)
    pg.all_reduce(s, op=pg.ReduceOp.SUM)
    return t.tolist(), s.tolist()


def cpu_info():
    """Host cores this process may use and the CPU model (lscpu's "Model name",
    else /proc/cpuinfo's first model line, else the machine type)."""
    import platform

    try:
        cores = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        cores = os.cpu_count()
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu model")):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"cores": cores, "cpu_count": os.cpu_count(), "model": model or platform.machine(),
            "reference_threads": 4 * (os.cpu_count() or 1),
            "threading": "the reference method starts 4 x std::thread::hardware_concurrency() OpenMP threads, "
                         "whatever the affinity mask"}


def cpu_reference_rate(U, ones, reps):
    """The reference's CPU method (oracle port: std::complex<double>, 4 x
    hardware threads, OpenMP) on the same input; returns (perm/s, cores, the
    method's value on this input)."""
    import oracle

    oracle.build.build(with_reference=False)
    oracle.port_permanent(U[:20, :20].copy(), ones[:20], ones[:20])  # warm the thread pool
    times = []
    val = None
    for _ in range(reps):
        t0 = time.perf_counter()
        val = oracle.port_permanent(U, ones, ones)
        times.append(time.perf_counter() - t0)
    return 1.0 / statistics.median(times), cpu_info()["cores"], complex(val)


def parity_record(got, want, pabs, against, single=False):
    """|gpu - want| against the contract's tolerance: max(1e-10 |perm|,
    1e-14 perm(|A|)) for complex128, max(1e-5 |perm|, 2^-23 perm(|A|)) for
    complex64."""
    rel, absf = (1e-5, 2.0 ** -23) if single else (1e-10, 1e-14)
    err = abs(complex(got) - complex(want))
    tol = max(rel * abs(want), absf * pabs)
    return {"against": against, "value": [float(np.real(want)), float(np.imag(want))], "abs_err": err,
            "rel_err": err / abs(want) if want else None, "tol": tol, "err_over_tol": err / tol,
            "pass": bool(err <= tol), "perm_abs": pabs}


def headline_config(n, dtype, world):
    """The config dict both arms print (identical for the same workload)."""
    return {"workload": "permanent n=%d %s, leading block of seeded %dx%d Haar unitary (seed 0), unit "
                        "multiplicities, one permanent per step" % (n, "complex128" if dtype == "c128" else
                                                                    "complex64", 2 * n, 2 * n),
            "n": n, "dtype": dtype, "parallelism": "replicas" if world > 1 else "1gpu",
            "l2": "GPU arm: L2 flushed before each timed step (a 256 MB write)"}


def run_reference(args, world, rank, pg):
    n = args.n
    if world > 1 and rank != 0:
        return
    U = haar_unitary(2 * n, 0)[:n, :n].copy()
    ones = np.ones(n, dtype=int)
    import oracle

    oracle.build.build(with_reference=False)
    for _ in range(args.warmup):
        oracle.port_permanent(U, ones, ones)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.port_permanent(U, ones, ones)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    info = cpu_info()
    line = {
        "impl": "reference",
        "metric": "permanents_per_second_n%d_complex128" % n,
        "value": value,
        "unit": "perm/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c128",
        "data": "synthetic (seeded Haar unitary)",
        "config": headline_config(n, "c128", world),
        "cpu_baseline": {"value": value, "unit": "perm/s", "cores": info["cores"], "kind": "port",
                         "model": info["model"], "threads": info["reference_threads"],
                         "sample": "%d full n=%d permanents, reference method (4 x hw threads)" % (args.steps, n)},
        "e2e": {"value": value, "unit": "perm/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def df_flops_per_step(n):
    """FP32 flops one all-ones double-float step executes (FMA = 2), counted
    from the kernel: 10 per column sum (two exact grid sums of five adds), 44
    per complex double-float product (two real parts of 22: two products, two
    FMA error terms, a TwoSum, four FMA cross terms), n - 1 products (two
    chains and their join), 38 for the weighted double-float accumulation."""
    return 10.0 * n + 44.0 * (n - 1) + 38.0


def time_calls(pg_engine, torch, flush, U, ones, steps, mode):
    """Per-step engine timings of `steps` public-API calls (host buffers in,
    host result out), L2 flushed before each call."""
    dev, walk, e2e = [], [], []
    tm = None
    res = None
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if mode == "api":
            res = pg_engine.permanent(U, ones, ones)
        else:
            res = pg_engine.permanent_dd(U, ones, ones, mode=mode)[0]
        e2e.append(time.perf_counter() - t0)
        tm = pg_engine.last_timing()
        dev.append(tm["device_ms"])
        walk.append(tm["walk_ms"])
    return dev, walk, e2e, tm, res


def bench_config2(pg_engine, torch, flush, peaks, cpu=True):
    """Single large permanents, n = 24, 26, 28, 30: the leading n x n block of
    a seeded 2n x 2n Haar unitary (seed 0), unit multiplicities, one
    permanent per launch over all SMs, in the three arithmetics -- the
    double-float walk (the complex128 default), the FP64 walk and the
    complex64 walk.  Per entry: perm/s (device time of the pipeline, L2
    flushed before each call), the walk's fraction of the measured FP32 or
    FP64 peak, and the result's error against the double-double oracle
    (n = 24) or the reference's CPU method (n >= 26), with the contract's
    tolerance; the reference method's perm/s on the host cores beside it."""
    import oracle

    oracle.build.build(with_reference=False)
    out = {"workload": "leading n x n block of Haar(2n) seed 0, unit multiplicities, one permanent per launch",
           "entries": {}}
    reps = {24: 8, 26: 5, 28: 3, 30: 2}
    all_pass = True
    for n in (24, 26, 28, 30):
        U = haar_unitary(2 * n, 0)[:n, :n].copy()
        ones = np.ones(n, dtype=int)
        U64 = U.astype(np.complex64)
        F = flops_all_ones(n)
        row = {}
        if cpu:
            t0 = time.perf_counter()
            port_val = complex(oracle.port_permanent(U, ones, ones))
            cpu_s = time.perf_counter() - t0
            pabs = float(abs(oracle.port_permanent(np.abs(U).astype(np.complex128), ones, ones)))
            if n <= 24:
                against = "double-double oracle"
                ref = oracle.permanent(U, ones, ones)
                ref64 = oracle.permanent(U64.astype(np.complex128), ones, ones)
            else:
                against = "reference CPU method (oracle port)"
                ref = port_val
                ref64 = complex(oracle.port_permanent(U64.astype(np.complex128), ones, ones))
            row["cpu_reference"] = {"value": 1.0 / cpu_s, "unit": "perm/s", "cores": cpu_info()["cores"],
                                    "kind": "port", "sample": "one full n=%d complex128 permanent" % n}
        for arith in ("df", "fp64", "c64"):
            A = U64 if arith == "c64" else U
            mode = "api" if arith == "c64" else arith
            time_calls(pg_engine, torch, flush, A, ones, 1, mode)  # first use of the instantiation
            dev, walk, _, _, res = time_calls(pg_engine, torch, flush, A, ones, reps[n], mode)
            w = statistics.mean(walk) / 1e3
            rec = {"value": len(dev) / (sum(dev) / 1e3), "unit": "perm/s", "walk_ms": 1e3 * w}
            if arith == "df":
                rec["achieved_tflops"] = 2.0 ** (n - 1) * df_flops_per_step(n) / w / 1e12
                rec["peak_tflops"] = peaks["fp32_tflops"]
                rec["basis"] = "FP32 flops executed by the double-float walk, 2^(n-1)(54n-6), vs measured FP32 peak"
                rec["complex128_algorithmic_tflops"] = F / w / 1e12
            elif arith == "fp64":
                rec["achieved_tflops"] = F / w / 1e12
                rec["peak_tflops"] = peaks["fp64_tflops"]
                rec["basis"] = "algorithmic 2^(n-1)(10n+4) vs measured FP64 peak"
            else:
                rec["achieved_tflops"] = F / w / 1e12
                rec["peak_tflops"] = peaks["fp32_tflops"]
                rec["basis"] = "algorithmic 2^(n-1)(10n+4) vs measured FP32 peak"
            rec["frac"] = rec["achieved_tflops"] / rec["peak_tflops"]
            if cpu:
                rec["parity"] = parity_record(res, ref64 if arith == "c64" else ref, pabs, against,
                                              single=arith == "c64")
                all_pass = all_pass and rec["parity"]["pass"]
                rec["speedup_vs_cpu"] = rec["value"] / row["cpu_reference"]["value"]
            row["complex64" if arith == "c64" else ("complex128_df" if arith == "df" else "complex128_fp64")] = rec
        out["entries"]["n%d" % n] = row
    if cpu:
        out["all_within_tolerance"] = all_pass
    return out


def bench_tuning(reps=5):
    """Tuned against default on the benchmarked shapes: the n = 28 headline
    permanent, the 4096-pattern batch (one graph-captured plan), a Metropolis
    block of 8192 complex64 target permanents, and the exact sampler's last
    photon step.  Each is timed (median device time of `reps` graph
    executions) with the engine's tuning table emptied (the defaults) and
    with the table the package loaded (the autotuner's cache for this GPU and
    library version)."""
    from piquasso_gb300 import _lib, autotune

    lib = _lib.load()
    key = autotune.cache_key(lib)
    entries = autotune.cached_entries(key)
    out = {"cache_key": key, "cache_entries": len(entries),
           "how": "median device ms of %d executions of one graph-captured plan per setting" % reps}
    names = ("single_n28_df", "batch_4096_d40_n20", "target_8192_n24_d48", "sampler_last_step_2048_n24_d48")
    ws = {w.name: w for w in autotune.standard_workloads()}
    for name in names:
        w = ws[name]
        lib.pqg_tuning_clear()
        d_ms, _ = autotune.time_workload(w, autotune.DEFAULT_SETTINGS, reps)
        autotune.install(entries, lib)
        t_ms, _ = autotune.time_workload(w, autotune.DEFAULT_SETTINGS, reps)
        with w.plan() as p:
            import ctypes

            v = [ctypes.c_int64(0) for _ in range(3)]
            b = ctypes.c_int32(0)
            lib.pqg_plan_config(p._h, *[ctypes.byref(x) for x in v], ctypes.byref(b))
        out[name] = {"default_ms": d_ms, "tuned_ms": t_ms, "speedup": d_ms / t_ms,
                     "tuned_settings": {"items_per_smsp": v[0].value, "p_max": v[1].value,
                                        "seed_steps": v[2].value, "blocks_per_sm": b.value}}
    return out


def batch_workload():
    """4096 output patterns drawn uniformly from the compositions of 20 photons
    into 40 modes with at most 4 per mode; seeded 40x40 Haar unitary; one
    photon in each of modes 0..19."""
    from piquasso_gb300 import workloads

    U = workloads.haar_unitary(40, 1)
    inp = np.array([1] * 20 + [0] * 20)
    pats = workloads.capped_compositions(20, 40, 4, 4096, seed=1)
    return U, inp, pats


def bench_batch(pg_engine, torch, flush, args, cpu=True):
    """Batched probabilities: one plan, executed as one CUDA graph per step."""
    U, inp, pats = batch_workload()
    plan = pg_engine.PermanentPlan(U, pats, inp)
    info = plan.info()
    for _ in range(2):
        plan.run()
    ms = []
    for _ in range(max(3, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        plan.launch()
        ms.append(plan.synchronize())
    vals = plan.read()
    plan.close()
    # end to end through the public batch call (planning and copies included)
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        v2 = pg_engine.permanent_batch(U, pats, inp)
    e2e_s = (time.perf_counter() - t0) / reps
    out = {"value": len(pats) / (statistics.mean(ms) / 1e3), "unit": "perm/s",
           "graph_ms": statistics.mean(ms), "e2e": {"value": len(pats) / e2e_s, "unit": "perm/s"},
           "gray_steps": info["steps"], "algorithmic_tflops": info["flops"] / (statistics.mean(ms) / 1e3) / 1e12,
           "max_rel_diff_e2e_vs_graph": float(np.max(np.abs(v2 - vals) / np.abs(vals))),
           "workload": "4096 uniform capped compositions (n=20, d=40, <= 4 per mode), seeded Haar(40), "
                       "complex128 (double-float walk), one graph-captured launch"}
    if cpu:
        import oracle

        k = 256
        t0 = time.perf_counter()
        for p in pats[:k]:
            oracle.port_permanent(U, p, inp)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": k / dt, "unit": "perm/s", "cores": cpu_info()["cores"], "kind": "port",
                               "sample": "first %d of the 4096 patterns, one reference-method call each" % k}
    return out


def bench_sampling(args):
    """Boson sampling at n=24 photons in d=48 modes (seeded Haar(48), seed 3,
    one photon in each of modes 0..23): the exact GPU sampler against the
    learned-proposal Metropolis sampler (1024 chains, the shipped network) and
    the same Metropolis sampler without the network; two-mode-marginal TVD
    against the exact marginals on 16 random mode pairs."""
    import os as _os

    from piquasso_gb300 import marginals, metropolis, proposal, sampling, workloads

    U = workloads.haar_unitary(48, 3)
    inp = np.array([1] * 24 + [0] * 24)
    out = {"workload": "n=24, d=48, Haar(48) seed 3, inputs in modes 0..23; complex64 permanents"}
    res = {}
    have = _os.path.exists(proposal.DEFAULT_WEIGHTS)
    mlp = proposal.load_mlp() if have else None
    runs = (("metropolis_learned", dict(mlp=mlp)),) if have else ()
    runs += (("metropolis_no_network", dict(baseline=True)),)
    pairs = None
    for name, kw in runs:
        r = metropolis.evaluate(U, inp, chains=1024, steps=args.mcmc_steps, burn_in=30, seed=4, **kw)
        pairs = [tuple(p) for p in r.pop("pairs")]
        res[name] = r
    tm = {}
    S = sampling.generate_samples_batched(inp, args.exact_samples, U.astype(np.complex64), 21, batch_size=4096,
                                          timings=tm)
    tv = marginals.tvd_two_mode(S, inp, U, pairs)
    res["exact"] = {"samples_per_s": args.exact_samples / tm["total_s"], "tvd_mean": float(tv.mean()),
                    "tvd_max": float(tv.max()), "samples": args.exact_samples, **tm}
    for name in res:
        if name != "exact":
            res[name]["speedup_vs_exact"] = res[name]["samples_per_s"] / res["exact"]["samples_per_s"]
    out.update(res)
    return out


def bench_training(args):
    """Training throughput of the learned proposal on the engine's kernels
    (tcgen05 GEMMs, softmax cross-entropy, bias gradients, Adam): Adam steps
    on batches of 65536 feature rows (synthetic features and targets of the
    training shapes: 16 features, occupations 0..7), plus the forward GEMM of
    a hidden layer (65536 x 256 x 256, bias + GELU epilogue) timed alone."""
    import ctypes

    import torch

    from piquasso_gb300 import _lib, proposal

    rows = 65536
    g = torch.Generator(device="cuda").manual_seed(0)
    X = torch.randn(rows, proposal.F, device="cuda", generator=g).to(torch.bfloat16)
    hi = torch.full((rows,), proposal.CAP, dtype=torch.int8, device="cuda")
    lo = torch.zeros(rows, dtype=torch.int8, device="cuda")
    tgt = torch.randint(0, proposal.CLASSES, (rows,), device="cuda", generator=g).to(torch.int8)
    mlp = proposal.MLP(seed=0)
    for _ in range(3):
        loss, gW, gb = mlp.loss_and_grads(X, lo, hi, tgt)
        mlp.adam(gW, gb)
    steps = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        loss, gW, gb = mlp.loss_and_grads(X, lo, hi, tgt)
        mlp.adam(gW, gb)
    e1.record()
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1) / steps
    L = _lib.load()
    A = torch.randn(rows, 256, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.empty(rows, 256, device="cuda")
    Cb = torch.empty(rows, 256, device="cuda", dtype=torch.bfloat16)
    fp = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float))  # noqa: E731
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    times = []
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > L2 (129 MB): cold operands
    for _ in range(8):
        flush.zero_()
        e0.record()
        st = L.pqg_mlp_gemm_tc(vp(A), 256, vp(mlp.WbT[1]), 256, rows, 256, 256, 1, fp(C), vp(Cb), fp(mlp.b[1]),
                               None, None, 0, None)
        e1.record()
        torch.cuda.synchronize()
        assert st == 0
        times.append(e0.elapsed_time(e1))
    gms = float(np.median(times[3:]))
    flops = 2.0 * rows * 256 * 256
    moved = rows * 256 * 2 + 256 * 256 * 2 + rows * 256 * (4 + 2)
    return {"workload": "Adam steps on 65536-row batches of the 16->256->256->256->8 MLP (BF16, FP32 accumulation)",
            "step_ms": step_ms, "rows_per_s": rows / (step_ms * 1e-3),
            "forward_gemm": {"shape": [rows, 256, 256], "ms": gms, "tflops": flops / (gms * 1e-3) / 1e12,
                             "gb_per_s": moved / (gms * 1e-3) / 1e9,
                             "hbm_frac": moved / (gms * 1e-3) / 1e9 / hbm_gbs() if hbm_gbs() else None,
                             "l2": "flushed before each launch (256 MB write)",
                             "kernel": "persistent (65536 rows >= 2 x SMs tiles): B resident, two TMEM accumulators, TMA tensor-store epilogue",
                             "note": "memory-bound at this shape: 64 flop/byte of operands and outputs"}}


def bench_next_rows(args, cpu=True):
    """The rows beyond the permanent: the permanent gradient (n=20, one
    Laplace walk per row, against the reference's n^2 minors through the
    reference CPU method on a sample of them), exact marginals on four and
    five modes at n=24 (the five-mode program holds about 89 GB of degree
    blocks in HBM), and the lossy sampler's throughput."""
    import piquasso_gb300 as pge
    from piquasso_gb300 import marginals, sampling, workloads

    out = {}
    n = 20
    A = haar_unitary(2 * n, 1)[:n, :n].copy()
    o = np.ones(n, dtype=int)
    pge.permanent_grad(A, o, o)
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        G = pge.permanent_grad(A, o, o)
        ts.append(time.perf_counter() - t0)
    g = {"workload": "gradient of the n=20 all-ones permanent (complex128), leading block of Haar(40) seed 1",
         "ms": 1e3 * statistics.median(ts), "entries": n * n}
    if cpu:
        import oracle

        oracle.build.build(with_reference=False)
        k = 8
        t0 = time.perf_counter()
        for j in range(k):  # entries (0, j): rows - e_0, cols - e_j, the reference's per-entry minor
            r2, c2 = o.copy(), o.copy()
            r2[0] -= 1
            c2[j] -= 1
            v = oracle.port_permanent(A, r2, c2)
            assert abs(v - G[0, j]) <= 1e-9 * abs(G).max()
        per = (time.perf_counter() - t0) / k
        g["cpu_baseline"] = {"ms": 1e3 * per * n * n, "unit": "ms per gradient", "cores": cpu_info()["cores"],
                             "kind": "port", "sample": "%d of the %d minors (reference method), scaled" % (k, n * n)}
        g["speedup_vs_cpu"] = g["cpu_baseline"]["ms"] / g["ms"]
    out["gradient_n20"] = g
    U = workloads.haar_unitary(48, 3)
    inp = np.array([1] * 24 + [0] * 24)
    for k in (4, 5):
        modes = tuple(range(k))
        t0 = time.perf_counter()
        p = marginals.marginal(inp, U, modes)
        dt = time.perf_counter() - t0
        out["marginal_k%d_n24" % k] = {"workload": "exact %d-mode marginal, n=24, d=48, Haar(48) seed 3" % k,
                                        "s": dt, "outcomes": int(p.size), "sum": float(p.sum())}
    tm = {}
    S = sampling.generate_samples_batched(inp, 8192, U.astype(np.complex64), 5, batch_size=8192, timings=tm,
                                          transmission=0.5)
    out["lossy_sampler_n24_d48"] = {"workload": "uniform loss T=0.5, n=24 inputs, d=48, batched, complex64",
                                    "samples_per_s": 8192 / tm["total_s"], "mean_photons": float(S.sum(1).mean())}
    return out


def run_ours(args, world, rank, local, pg):
    import __graft_entry__

    __graft_entry__.build_engine()
    import piquasso_gb300 as pg_engine
    import torch

    torch.cuda.set_device(local)
    n = args.n
    U128 = haar_unitary(2 * n, 0)[:n, :n].copy()
    ones = np.ones(n, dtype=int)
    U = U128.astype(np.complex64) if args.dtype == "c64" else U128
    peaks = pg_engine.measure_vector_peaks(20.0)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > L2 (129 MB)

    with ClockSampler(local) as clk:
        for _ in range(args.warmup):  # the timed steps' work, flush included
            flush.zero_()
            pg_engine.permanent(U, ones, ones)
        torch.cuda.synchronize()
        if pg is not None:
            pg.barrier()
        launches0 = pg_engine.kernel_launches()
        clk.start_region()
        t_region = time.perf_counter()
        dev_ms, walk_ms, e2e_s, tm, result = time_calls(pg_engine, torch, flush, U, ones, args.steps, "api")
        torch.cuda.synchronize()
        region = time.perf_counter() - t_region
    launches = pg_engine.kernel_launches() - launches0
    clocks = clk.summary()
    h2d, d2h = tm["h2d_bytes"], tm["d2h_bytes"]

    total_dev = sum(dev_ms) / 1e3
    total_e2e = sum(e2e_s)
    (max_dev, max_e2e), _ = allreduce_max_sum(pg, [total_dev, total_e2e], [0.0])
    value = world * args.steps / max_dev
    e2e = world * args.steps / max_e2e
    mean_walk_s = statistics.mean(walk_ms) / 1e3
    F = flops_all_ones(n)

    if args.dtype == "c64":
        roof = {"bound": "fp32", "achieved": F / mean_walk_s / 1e12, "peak": peaks["fp32_tflops"],
                "unit": "TFLOP/s", "flops_per_launch": F,
                "flops_basis": "algorithmic 2^(n-1)(10n+4), complex64 walk on the FP32 pipes"}
    else:
        # the default complex128 path: double-float walk on the FP32 pipes
        Fdf = 2.0 ** (n - 1) * df_flops_per_step(n)
        roof = {"bound": "fp32", "achieved": Fdf / mean_walk_s / 1e12, "peak": peaks["fp32_tflops"],
                "unit": "TFLOP/s", "flops_per_launch": Fdf,
                "flops_basis": "FP32 flops the double-float walk executes, 2^(n-1)(54n-6) (FMA = 2)",
                "complex128_algorithmic_tflops": F / mean_walk_s / 1e12}
    roof["frac"] = roof["achieved"] / roof["peak"]
    # DRAM bytes (read + write) of one headline launch: a recorded constant
    # from one ncu capture of this workload (the walk reads the 12.5 KB
    # matrix's prefix tables, seeds and weight tables, and writes its
    # partials); a bench run cannot read DRAM counters itself
    if n == 28 and args.dtype == "c128":
        roof["traffic"] = TRAFFIC_N28_DF
        roof["traffic_source"] = ("recorded constant, not measured by this run: ncu dram__bytes_read.sum + "
                                  "dram__bytes_write.sum of one n=28 double-float walk launch, captured %s"
                                  % TRAFFIC_N28_DF_DATE)
    else:
        roof["traffic"] = None
    roof["peak_source"] = "measured: engine FMA-chain microkernel (pqg_measure_vector_peaks)"
    roof["walk_ms"] = 1e3 * mean_walk_s

    line = {
        "metric": "permanents_per_second_n%d_%s" % (n, "complex128" if args.dtype == "c128" else "complex64"),
        "value": value,
        "unit": "perm/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * max_dev / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": args.dtype,
        "data": "synthetic (seeded Haar unitary)",
        "config": headline_config(n, args.dtype, world),
        "timing": {"l2": "flushed between steps (256 MB write)",
                   "c128_arithmetic": "auto (double-float walk, FP64 seeds and double-double sums)"},
        "e2e": {"value": e2e, "unit": "perm/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": roof,
        "peaks_measured": peaks,
        "gpu_launches": launches,
        "clocks": clocks,
        "result": [float(np.real(result)), float(np.imag(result))],
        "timed_region_s": region,
    }
    if args.dtype == "c128" and not args.no_variants:
        # the FP64 walk against the FP64 peak, and the complex64 walk
        dev, walk, _, _, r64 = time_calls(pg_engine, torch, flush, U128, ones, max(3, args.steps // 4), "fp64")
        w = statistics.mean(walk) / 1e3
        line["fp64_walk"] = {"value": len(dev) / (sum(dev) / 1e3), "unit": "perm/s",
                             "achieved_tflops": F / w / 1e12, "peak_fp64_tflops": peaks["fp64_tflops"],
                             "frac": F / w / 1e12 / peaks["fp64_tflops"],
                             "flops_basis": "algorithmic 2^(n-1)(10n+4)",
                             "abs_diff_vs_default": abs(complex(r64) - complex(result))}
        U64 = U128.astype(np.complex64)
        dev, walk, _, _, r32 = time_calls(pg_engine, torch, flush, U64, ones, max(3, args.steps // 4), "api")
        w = statistics.mean(walk) / 1e3
        line["complex64_walk"] = {"value": len(dev) / (sum(dev) / 1e3), "unit": "perm/s",
                                  "achieved_tflops": F / w / 1e12, "peak_fp32_tflops": peaks["fp32_tflops"],
                                  "frac": F / w / 1e12 / peaks["fp32_tflops"],
                                  "rel_diff_vs_default": abs(complex(r32) - complex(result)) / abs(complex(result))}
    def section(fn, *a, **kw):
        # a secondary line that fails records its error instead of taking
        # the headline line down with it
        try:
            return fn(*a, **kw)
        except Exception as e:  # noqa: BLE001
            return {"error": "%s: %s" % (type(e).__name__, e)}

    if not args.no_variants:
        line["batch_4096_d40_n20"] = section(bench_batch, pg_engine, torch, flush, args,
                                             cpu=(rank == 0 and not args.no_cpu_baseline))
    if not args.no_variants and not args.no_sampling:
        line["sampling_n24_d48"] = section(bench_sampling, args)
        line["training_mlp"] = section(bench_training, args)
        line["next_rows"] = section(bench_next_rows, args, cpu=(rank == 0 and not args.no_cpu_baseline))
    if rank == 0 and not args.no_variants:
        line["config2"] = section(bench_config2, pg_engine, torch, flush, peaks, cpu=not args.no_cpu_baseline)
        line["tuning"] = section(bench_tuning)
    if rank == 0 and not args.no_cpu_baseline:
        rate, cores, ref_val = cpu_reference_rate(U128, ones, reps=args.cpu_reps)
        info = cpu_info()
        line["cpu_baseline"] = {"value": rate, "unit": "perm/s", "cores": cores, "kind": "port",
                                "model": info["model"], "threads": info["reference_threads"],
                                "sample": "median of %d full n=%d complex128 permanents, reference method, "
                                          "4 x hw threads" % (args.cpu_reps, n)}
        if args.dtype == "c128":
            import oracle

            pabs = float(abs(oracle.port_permanent(np.abs(U128).astype(np.complex128), ones, ones)))
            par = {"reference_method": parity_record(result, ref_val, pabs, "reference CPU method (oracle port)")}
            if not args.no_dd_oracle:
                t0 = time.perf_counter()
                par["dd_oracle"] = parity_record(result, oracle.permanent(U128, ones, ones), pabs,
                                                 "double-double oracle")
                par["dd_oracle"]["oracle_s"] = time.perf_counter() - t0
            par["pass"] = all(v["pass"] for v in par.values() if isinstance(v, dict))
            par["tolerance"] = "max(1e-10 |perm|, 1e-14 perm(|A|)); perm(|A|) by the reference method"
            line["parity"] = par
    if rank == 0:
        print(json.dumps(line), flush=True)


def profile_case(name):
    """Small named cases for ncu captures (no JSON line): each runs its kernel
    a few times after building the engine.
      gemm16k    — the tcgen05 forward GEMM, 16384 x 256 x 256, bias + GELU, 6 launches
                   (one 128-row tile per CTA);
      gemm65k    — the same at 65536 rows, the benchmarked shape (the persistent kernel);
      target1024 — 1024 complex64 permanents of learned-proposal patterns at
                   n=24, d=48 (one Metropolis block's targets), 3 calls;
      laplace24  — 1024 complex64 Laplace permanents shaped like the exact
                   sampler's last photon step at n=24, d=48, 3 calls;
      df24       — one n=24 complex128 permanent (double-float walk), 4 calls;
      df28       — the n=28 headline permanent (double-float walk), 3 calls;
      propose8192 — the fused tensor-core proposal step for 8192 chains at
                   n=24, d=48 (48 launches per draw): one eager draw, then 3
                   graph replays;
      draw2048   — the exact sampler's fused step (Laplace permanents + pmf +
                   draw) for 2048 shots after 16 photons at n=24, d=48, 3 calls;
      laplace24c128 — laplace24 in complex128 (the double-float Laplace walk);
      train65k   — Adam steps of the learned proposal on a 65536-row batch
                   (forward, backward, bias gradients, Adam), 4 steps."""
    import ctypes

    import __graft_entry__

    __graft_entry__.build_engine()
    import torch

    import piquasso_gb300 as pge
    from piquasso_gb300 import _lib, metropolis, proposal, workloads

    if name in ("gemm16k", "gemm65k"):
        L = _lib.load()
        rows = 16384 if name == "gemm16k" else 65536
        g = torch.Generator(device="cuda").manual_seed(0)
        A = torch.randn(rows, 256, device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn(256, 256, device="cuda", generator=g).to(torch.bfloat16)
        bias = torch.zeros(256, device="cuda")
        C = torch.empty(rows, 256, device="cuda")
        Cb = torch.empty(rows, 256, device="cuda", dtype=torch.bfloat16)
        fp = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float))  # noqa: E731
        vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        for _ in range(6):
            assert L.pqg_mlp_gemm_tc(vp(A), 256, vp(B), 256, rows, 256, 256, 1, fp(C), vp(Cb), fp(bias), None, None,
                                     0, None) == 0
        torch.cuda.synchronize()
    elif name == "train65k":
        rows = 65536
        g = torch.Generator(device="cuda").manual_seed(0)
        X = torch.randn(rows, proposal.F, device="cuda", generator=g).to(torch.bfloat16)
        hi = torch.full((rows,), proposal.CAP, dtype=torch.int8, device="cuda")
        lo = torch.zeros(rows, dtype=torch.int8, device="cuda")
        tgt = torch.randint(0, proposal.CLASSES, (rows,), device="cuda", generator=g).to(torch.int8)
        mlp = proposal.MLP(seed=0)
        for _ in range(4):
            loss, gW, gb = mlp.loss_and_grads(X, lo, hi, tgt)
            mlp.adam(gW, gb)
        torch.cuda.synchronize()
    elif name == "target1024":
        U = workloads.haar_unitary(48, 3)
        inp = np.array([1] * 24 + [0] * 24)
        ps = metropolis.ProposalSampler(proposal.load_mlp(), proposal.ModeStats(U, inp), 1024)
        y, _ = ps.propose(seed=11)
        pats = y.cpu().numpy().astype(np.int64)
        for _ in range(3):
            pge.permanent_batch(U.astype(np.complex64), pats, inp)
    elif name in ("laplace24", "laplace24c128"):
        # the exact sampler's last photon step at n=24, d=48: 1024 shots with 23
        # photons placed (exact samples less one photon), 24 input columns
        from piquasso_gb300 import sampling

        U = workloads.haar_unitary(48, 3)
        inp = np.array([1] * 24 + [0] * 24)
        S = sampling.generate_samples_batched(inp, 1024, U.astype(np.complex64), 7)
        rng = np.random.default_rng(1)
        rows = S.copy()
        for s_ in range(len(rows)):
            nz = np.nonzero(rows[s_])[0]
            rows[s_, nz[rng.integers(len(nz))]] -= 1
        cols = np.broadcast_to(inp, rows.shape)
        dt = np.complex64 if name == "laplace24" else np.complex128
        for _ in range(3):
            pge.permanent_laplace_batch(U.astype(dt), rows, cols)
    elif name == "propose8192":
        U = workloads.haar_unitary(48, 3)
        inp = np.array([1] * 24 + [0] * 24)
        ps = metropolis.ProposalSampler(proposal.load_mlp(), proposal.ModeStats(U, inp), 8192)
        for s_ in range(4):  # the first call runs eagerly and captures the graph
            ps.propose(seed=s_)
        torch.cuda.synchronize()
    elif name == "draw2048":
        from piquasso_gb300 import sampling

        U = workloads.haar_unitary(48, 3).astype(np.complex64)
        inp = np.array([1] * 24 + [0] * 24)
        # 2048 shots with 16 photons placed: exact samples of the first 16 inputs
        rows = sampling.generate_samples_batched(np.array([1] * 16 + [0] * 32), 2048, U, 5)
        rng = np.random.default_rng(2)
        cols = np.zeros_like(rows)
        for s_ in range(len(cols)):
            cols[s_, rng.permutation(24)[:17]] = 1
        u = rng.random(len(rows))
        for _ in range(3):
            pge.sampler_step_batch(U, rows, cols, u)
    elif name == "df28":
        A = haar_unitary(56, 0)[:28, :28].copy()
        for _ in range(3):
            pge.permanent(A, np.ones(28, int), np.ones(28, int))
    elif name == "df24":
        A = haar_unitary(48, 0)[:24, :24].copy()
        for _ in range(4):
            pge.permanent(A, np.ones(24, int), np.ones(24, int))
    else:
        raise SystemExit("unknown profile case %r" % name)
    print(json.dumps({"profile_case": name, "timing": pge.last_timing()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=28)
    ap.add_argument("--dtype", choices=["c128", "c64"], default="c128")
    ap.add_argument("--cpu-reps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-sampling", action="store_true")
    ap.add_argument("--no-dd-oracle", action="store_true", help="skip the double-double check of the headline")
    ap.add_argument("--mcmc-steps", type=int, default=600)
    ap.add_argument("--exact-samples", type=int, default=32768)
    ap.add_argument("--profile-case", default=None, help="run one small named case for ncu and exit")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        run_ours(args, world, rank, local, pg)


if __name__ == "__main__":
    main()
