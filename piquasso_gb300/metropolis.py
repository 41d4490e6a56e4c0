"""Independence Metropolis boson sampling with a learned proposal.

B chains run in lock step.  Every step draws B proposals y from the
autoregressive MLP (proposal.py) on the device — features, network and draw
for one output mode at a time — together with their exact log q(y), and
accepts y over the chain state x with probability

    min(1, p(y) q(x) / (p(x) q(y))),   p(y) = |Per(U[y, in])|^2 / prod_i y_i!

(the output probability of ideal boson sampling with single-photon inputs,
as in the reference's passive/utils.py:131-138 and probabilities.py:26-54).
The target probabilities come from one batched complex64 permanent launch per
block of steps (FP32 products with FP64-class seeds and double-double sums),
overlapped with the drawing of the next block (see run_chains).  Patterns
with a mode holding more than 7 photons cannot be proposed: the chain samples
the target restricted to occupations <= 7, whose distance from the exact
distribution the two-mode-marginal TVD against the exact marginals measures.

`baseline=True` replaces the network by the exact one-mode marginals
(logits log p_j(k)): the same sampler without the learned part.
"""

import ctypes
import time
from math import lgamma

import numpy as np

from . import _lib
from .permanent import permanent_batch
from .proposal import CAP, CLASSES, F, LD, ModeStats


def _fp(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float))


def _i8(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_int8))


def _i32(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_int32))


class ProposalSampler:
    """Draws B patterns and their log q on the device."""

    def __init__(self, mlp, stats: ModeStats, B, baseline=False, device="cuda", fused=True):
        import torch

        self.torch = torch
        self.mlp = mlp
        self.stats = stats
        self.B = B
        self.d = stats.d
        self.n = stats.n
        self.baseline = baseline
        ms = np.zeros((self.d, 12), dtype=np.float32)
        ms[:, :5] = stats.p
        ms[:, 5] = stats.tail
        ms[:, 6] = stats.mu
        ms[:, 7] = stats.var
        ms[:, 8] = stats.mu_suffix[: self.d]
        self.ms = torch.from_numpy(ms).to(device)
        self.C = torch.from_numpy(stats.C.astype(np.float32)).to(device)
        self.X = torch.zeros(B, F, dtype=torch.bfloat16, device=device)
        self.lo = torch.zeros(B, dtype=torch.int8, device=device)
        self.hi = torch.zeros(B, dtype=torch.int8, device=device)
        self.samples = torch.zeros(B, self.d, dtype=torch.int8, device=device)
        self.n_rem = torch.zeros(B, dtype=torch.int32, device=device)
        self.shift = torch.zeros(B, self.d, dtype=torch.float32, device=device)
        self.logq = torch.zeros(B, dtype=torch.float32, device=device)
        self.seed_dev = torch.zeros(1, dtype=torch.int64, device=device)
        self.graph = None
        # one fused tensor-core kernel per mode (pqg_proposal_step_tc) unless
        # asked for the separate feature / GEMM / sampling kernels
        self.fused = bool(fused) and not baseline
        if baseline:
            # exact one-mode marginals; the tail mass spread over occupations 5..7
            lg = np.zeros((self.d, LD), dtype=np.float32)
            lg[:, :5] = np.log(np.maximum(stats.p, 1e-30))
            lg[:, 5:] = np.log(np.maximum(stats.tail / 3.0, 1e-30))[:, None]
            self.base_logits = torch.from_numpy(lg).to(device)

    def propose(self, seed):
        """Draws the B patterns for `seed`: (samples int8 (B, d), logq (B,)),
        the sampler's own device buffers (copy them before the next call).

        The whole autoregressive draw (d rounds of features, the MLP and the
        sampling kernel) is captured once as a CUDA graph and replayed with
        the seed in device memory: hundreds of small launches become one."""
        torch = self.torch
        if self.graph is None:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self._draw_rounds()  # first use: kernel attributes, allocations
            torch.cuda.current_stream().wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._draw_rounds()
            self.graph = g
        v = int(seed) % (1 << 64)  # the bits of the uint64 seed, stored as int64
        self.seed_dev.fill_(v - (1 << 64) if v >= (1 << 63) else v)
        self.graph.replay()
        if self.fused:
            _lib.check_tc_status()  # (synchronises; the caller reads the draw at once anyway)
        return self.samples, self.logq

    def _draw_rounds(self):
        L = _lib.load()
        torch = self.torch
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.n_rem.fill_(self.n)
        self.shift.zero_()
        self.logq.zero_()
        B, d, n = self.B, self.d, self.n
        seed_ptr = ctypes.c_void_p(self.seed_dev.data_ptr())
        if self.fused:
            m = self.mlp
            w = [ctypes.c_void_p(t.data_ptr()) for t in m.WbT]
            for j in range(d):
                st = L.pqg_proposal_step_tc(j, B, d, n, _fp(self.ms), w[0], w[1], w[2], w[3], _fp(m.b[0]),
                                            _fp(m.b[1]), _fp(m.b[2]), _fp(m.b[3]), ctypes.c_uint64(0), seed_ptr,
                                            _i8(self.samples), _i32(self.n_rem), _fp(self.shift), _fp(self.C),
                                            _fp(self.logq), stream)
                if st:
                    raise RuntimeError(_lib.last_error())
            return
        for j in range(d):
            st = L.pqg_proposal_features(j, B, d, n, _fp(self.ms), _i32(self.n_rem), _fp(self.shift),
                                         ctypes.c_void_p(self.X.data_ptr()), _i8(self.lo), _i8(self.hi), stream)
            if st:
                raise RuntimeError(_lib.last_error())
            if self.baseline:
                logits = self.base_logits[j].expand(B, LD).contiguous()
            else:
                logits = self.mlp.forward(self.X, stream=stream)
            st = L.pqg_proposal_sample(j, B, d, _fp(logits), _i8(self.lo), _i8(self.hi), ctypes.c_uint64(0), seed_ptr,
                                       _i8(self.samples), _i32(self.n_rem), _fp(self.shift), _fp(self.C),
                                       _fp(self.ms), _fp(self.logq), stream)
            if st:
                raise RuntimeError(_lib.last_error())
        return self.samples, self.logq


def log_target(U64, patterns, inp):
    """log p(y) = log |Per(U[y, in])|^2 - sum log y!  for every row of patterns."""
    perms = permanent_batch(U64, patterns, inp)
    lf = np.array([lgamma(k + 1.0) for k in range(int(np.max(patterns)) + 2)])
    with np.errstate(divide="ignore"):
        return 2.0 * np.log(np.abs(perms).astype(np.float64)) - lf[patterns].sum(axis=1)


def run_chains(U, input_photons, mlp=None, chains=1024, steps=200, burn_in=50, seed=0, baseline=False,
               record=True, block=16):
    """Runs `chains` independent chains for `steps` steps; returns a dict with
    the recorded states (after burn-in), acceptance rate and timings.

    An independence proposal does not depend on the chain state, so the
    proposals of `block` consecutive steps are drawn as one batch of
    chains * block patterns and their target probabilities are one batched
    permanent launch.  Those launches run on two worker threads (the engine
    call releases the GIL and plans outside its lock), so one block's host
    planning overlaps the previous block's kernels while later blocks are
    drawn on the device; the accept/reject pass then walks each block's steps
    in order, exactly as a step-by-step chain would.  Proposal 0 of every
    chain is its initial state."""
    import torch
    from concurrent.futures import ThreadPoolExecutor

    inp = np.asarray(input_photons, dtype=int)
    U = np.asarray(U, dtype=np.complex128)
    U64 = U.astype(np.complex64)
    d = len(inp)
    block = max(1, int(block))
    stats = ModeStats(U, inp)
    sampler = ProposalSampler(mlp, stats, chains * block, baseline=baseline)
    rng = np.random.default_rng(seed)
    n_blocks = (steps + 1 + block - 1) // block
    t_prop = 0.0
    t_perm = [0.0]

    def draw(k):
        y_d, lq_d = sampler.propose(seed * 1000003 + 1 + k)
        y = y_d.cpu().numpy().astype(np.int64).reshape(block, chains, d)
        return y, lq_d.cpu().numpy().astype(np.float64).reshape(block, chains)

    def target(Y):
        t = time.perf_counter()
        lp = log_target(U64, Y.reshape(-1, d), inp).reshape(block, chains)
        t_perm[0] += time.perf_counter() - t  # summed over the two workers
        return lp

    from collections import deque

    sampler.propose(seed * 1000003)  # one-time setup outside the timing: captures the draw's CUDA graph
    t0 = time.perf_counter()
    accepted = 0
    proposals = 0
    kept = []
    x = logp_x = logq_x = None
    # two blocks' target launches in flight (one block's host planning
    # overlaps the other's kernels); proposals are drawn ahead on this thread
    with ThreadPoolExecutor(max_workers=2) as ex:
        inflight = deque()
        nxt = 0
        while nxt < min(2, n_blocks):
            ta = time.perf_counter()
            Yn, LQn = draw(nxt)
            t_prop += time.perf_counter() - ta
            inflight.append((Yn, LQn, ex.submit(target, Yn)))
            nxt += 1
        for k in range(n_blocks):
            Y, LQ, fut = inflight.popleft()
            if nxt < n_blocks:
                ta = time.perf_counter()
                Yn, LQn = draw(nxt)  # overlaps the workers' permanents
                t_prop += time.perf_counter() - ta
                inflight.append((Yn, LQn, ex.submit(target, Yn)))
                nxt += 1
            LP = fut.result()
            for s in range(block):
                g = k * block + s  # proposal index; 0 is the initial state
                if g > steps:
                    break
                if g == 0:
                    x, logp_x, logq_x = Y[0].copy(), LP[0].copy(), LQ[0].copy()
                    continue
                y, logp_y, logq_y = Y[s], LP[s], LQ[s]
                log_alpha = (logp_y - logp_x) - (logq_y - logq_x)
                acc = np.log(rng.random(chains)) < log_alpha
                x[acc] = y[acc]
                logp_x[acc] = logp_y[acc]
                logq_x[acc] = logq_y[acc]
                accepted += int(acc.sum())
                proposals += chains
                if record and g - 1 >= burn_in:
                    kept.append(x.copy())
    torch.cuda.synchronize()
    total = time.perf_counter() - t0
    out = {
        "acceptance": accepted / max(1, proposals),
        "chain_steps": proposals,
        "seconds": total,
        "samples_per_s": proposals / total,
        "propose_s": t_prop,
        "target_s": t_perm[0],
        "block": block,
    }
    if record:
        out["samples"] = np.concatenate(kept) if kept else np.zeros((0, len(inp)), dtype=np.int64)
    return out


def integrated_autocorrelation(series, c=5.0):
    """Integrated autocorrelation time of a scalar statistic recorded on
    several chains, ``series`` of shape (steps, chains): the normalised
    autocovariance rho_k averaged over the chains (about the overall mean),
    tau = 1 + 2 sum_{k=1}^{M} rho_k with Sokal's automatic window (the
    smallest M >= c tau(M)).  tau is 1 for independent draws; a chain of
    length T then holds about T / tau effective samples.  A constant
    statistic gives tau = 1."""
    x = np.asarray(series, dtype=np.float64)
    T = x.shape[0]
    x = x - x.mean()
    var = float(np.mean(x * x))
    if T < 2 or var == 0.0:
        return 1.0
    nfft = 1 << int(np.ceil(np.log2(2 * T)))
    f = np.fft.rfft(x, n=nfft, axis=0)
    acov = np.fft.irfft(f * np.conj(f), n=nfft, axis=0)[:T].sum(axis=1)
    acov /= (T - np.arange(T)) * x.shape[1]  # unbiased per lag, averaged over chains
    rho = acov / acov[0]
    tau = 1.0
    for m in range(1, T):
        tau += 2.0 * rho[m]
        if m >= c * tau:
            break
    return max(tau, 1.0)


def chain_autocorrelation(samples, chains):
    """tau of every mode's occupation, from recorded chain states in step-
    major order ((steps * chains, d), as run_chains records them); returns
    (max over modes, mean over modes)."""
    S = np.asarray(samples)
    steps = S.shape[0] // chains
    S = S[: steps * chains].reshape(steps, chains, -1)
    taus = [integrated_autocorrelation(S[:, :, j]) for j in range(S.shape[2])]
    return float(np.max(taus)), float(np.mean(taus))


def evaluate(U, input_photons, mlp=None, chains=1024, steps=300, burn_in=30, seed=0, baseline=False, pairs=None,
             pair_seed=0, n_pairs=16, block=16):
    """Samples/s, acceptance, two-mode-marginal TVD (mean and max over
    `pairs`, default `n_pairs` random mode pairs) and the chains' integrated
    autocorrelation time (mode occupations; the largest over the modes gives
    the effective samples per second) of one Metropolis run."""
    from .marginals import tvd_two_mode

    d = len(input_photons)
    if pairs is None:
        rng = np.random.default_rng(pair_seed)
        allp = [(a, b) for a in range(d) for b in range(a + 1, d)]
        pairs = [allp[i] for i in rng.choice(len(allp), size=min(n_pairs, len(allp)), replace=False)]
    out = run_chains(U, input_photons, mlp=mlp, chains=chains, steps=steps, burn_in=burn_in, seed=seed,
                     baseline=baseline, block=block)
    S = out.pop("samples")
    tv = tvd_two_mode(S, input_photons, U, pairs)
    tau_max, tau_mean = chain_autocorrelation(S, chains)
    out.update({"tvd_mean": float(tv.mean()), "tvd_max": float(tv.max()), "pairs": [list(p) for p in pairs],
                "kept_samples": chains * max(0, steps - burn_in), "tau_max": tau_max, "tau_mean": tau_mean,
                "effective_samples_per_s": out["samples_per_s"] / tau_max})
    return out
