"""Training the learned proposal by maximum likelihood on exact samples.

Exact samples come from the GPU exact sampler (sampling.generate_samples_batched)
for seeded Haar-random interferometers at n photons in d = 2n modes, one photon
in each of the first n modes; their exact probabilities come from batched
permanents and give the exact KL(p || q) = E_p[log p - log q] of the trained
proposal.  Training minimises the mean per-mode cross-entropy with Adam, on
the engine's BF16 tensor-core kernels.

Usage: python -m piquasso_gb300.train --out weights.npz [--samples-per-unitary N ...]
"""

import argparse
import json
import time

import numpy as np

from . import _lib, proposal, sampling, workloads
from .metropolis import log_target


def build_dataset(ns=(12, 13, 14, 15, 16), unitaries=4, samples_per_unitary=4096, seed=0, log=print):
    """Feature rows of exact samples: X (R, F) float32, lo, hi, target (R,) int8,
    plus per-unitary records for KL evaluation."""
    Xs, los, his, ts, recs = [], [], [], [], []
    for n in ns:
        d = 2 * n
        inp = np.array([1] * n + [0] * n)
        for u in range(unitaries):
            useed = 1000 * n + u + seed
            U = workloads.haar_unitary(d, useed)
            t0 = time.perf_counter()
            S = sampling.generate_samples_batched(inp, samples_per_unitary, U.astype(np.complex64), useed,
                                                  batch_size=samples_per_unitary)
            stats = proposal.ModeStats(U, inp)
            X, lo, hi, tgt = proposal.features(stats, S)
            keep = S.max(axis=1) <= proposal.CAP  # the proposal's support: occupations <= CAP
            Xs.append(X[keep].reshape(-1, proposal.F))
            los.append(lo[keep].reshape(-1))
            his.append(hi[keep].reshape(-1))
            ts.append(tgt[keep].reshape(-1))
            recs.append({"n": n, "U": U, "inp": inp, "samples": S[keep][:2048]})
            log("dataset n=%d unitary %d: %d samples (%d within the cap) in %.1f s"
                % (n, u, len(S), int(keep.sum()), time.perf_counter() - t0))
    return (np.concatenate(Xs), np.concatenate(los), np.concatenate(his), np.concatenate(ts)), recs


def evaluate_nll(mlp, X, lo, hi, target, d):
    """Mean negative log-likelihood per sample (nats) of rows grouped d per sample."""
    import torch

    Xb = torch.from_numpy(X).to("cuda", torch.bfloat16)
    lo_t = torch.from_numpy(lo).cuda()
    hi_t = torch.from_numpy(hi).cuda()
    tg = torch.from_numpy(target).cuda()
    loss, _, _ = mlp.loss_and_grads(Xb, lo_t, hi_t, tg)
    return float(loss.sum().item()) / (len(X) / d)


def kl_estimate(mlp, rec):
    """E_p[log p - log q] over the record's exact samples (nats)."""
    stats = proposal.ModeStats(rec["U"], rec["inp"])
    S = rec["samples"]
    X, lo, hi, tgt = proposal.features(stats, S)
    nll = evaluate_nll(mlp, X.reshape(-1, proposal.F), lo.reshape(-1), hi.reshape(-1), tgt.reshape(-1), stats.d)
    logp = log_target(rec["U"].astype(np.complex64), S, rec["inp"])
    return float(np.mean(logp)) + nll


def train(data, epochs=3, batch=65536, lr=2e-3, seed=0, log=print):
    import torch

    X, lo, hi, tgt = data
    mlp = proposal.MLP(seed=seed)
    Xd = torch.from_numpy(X).to("cuda", torch.bfloat16)
    lo_d = torch.from_numpy(lo).cuda()
    hi_d = torch.from_numpy(hi).cuda()
    tg_d = torch.from_numpy(tgt).cuda()
    R = len(X)
    g = torch.Generator(device="cuda").manual_seed(seed)
    history = []
    for ep in range(epochs):
        perm = torch.randperm(R, device="cuda", generator=g)
        tot, cnt = 0.0, 0
        t0 = time.perf_counter()
        for s in range(0, R - batch + 1, batch):
            idx = perm[s:s + batch]
            loss, gW, gb = mlp.loss_and_grads(Xd[idx], lo_d[idx], hi_d[idx], tg_d[idx])
            mlp.adam(gW, gb, lr=lr)
            tot += float(loss.mean().item())
            cnt += 1
        _lib.check_tc_status()
        history.append(tot / max(1, cnt))
        log("epoch %d: mean cross-entropy %.5f nats/mode (%.1f s)" % (ep, history[-1], time.perf_counter() - t0))
    return mlp, history


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--samples-per-unitary", type=int, default=4096)
    ap.add_argument("--unitaries", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    t0 = time.perf_counter()
    data, recs = build_dataset(unitaries=a.unitaries, samples_per_unitary=a.samples_per_unitary, seed=a.seed)
    t_data = time.perf_counter() - t0
    mlp, hist = train(data, epochs=a.epochs, seed=a.seed)
    kls = [kl_estimate(mlp, r) for r in recs[:: max(1, len(recs) // 5)]]
    sd = mlp.state_dict()
    np.savez(a.out, W0=sd["W"][0], W1=sd["W"][1], W2=sd["W"][2], W3=sd["W"][3], b0=sd["b"][0], b1=sd["b"][1],
             b2=sd["b"][2], b3=sd["b"][3], step=sd["step"])
    print(json.dumps({"rows": int(len(data[0])), "data_s": t_data, "train_s": time.perf_counter() - t0 - t_data,
                      "history": hist, "kl_nats": kls}))


if __name__ == "__main__":
    main()
