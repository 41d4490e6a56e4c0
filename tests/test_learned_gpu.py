"""GPU: the learned proposal — BF16 tensor-core MLP gradients against the CPU
oracle (oracle/mlp.py), parity of the device proposal's features and log q
with the training path, a Metropolis chain against exact marginals, and the
gain of the shipped (trained) network over the same sampler without it, on an
interferometer held out of training.

Tolerances: gradients and loss within 2e-2 relative (L2 norm) of the oracle,
which rounds to BF16 at the same points but accumulates in float64; proposal
log q within 1e-3 nats per pattern of the training-path log-likelihood (FP32
softmax, BF16 features built in two places).
"""

import numpy as np
import pytest

import oracle.mlp as omlp
from conftest import haar_unitary

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_mlp_gradients_match_oracle(engine):
    torch = pytest.importorskip("torch")
    from piquasso_gb300 import proposal

    rng = np.random.default_rng(0)
    M = 300  # not a multiple of the 64-row tile
    mlp = proposal.MLP(seed=3)
    for i in range(4):  # non-trivial biases
        mlp.b[i].copy_(torch.from_numpy(rng.normal(scale=0.1, size=mlp.b[i].shape).astype(np.float32)))
    X = rng.normal(size=(M, proposal.F)).astype(np.float32)
    hi = rng.integers(0, 5, size=M).astype(np.int8)
    lo = np.minimum(rng.integers(0, 3, size=M), hi).astype(np.int8)
    tgt = (lo + (rng.integers(0, 5, size=M) % (hi - lo + 1))).astype(np.int8)
    Xb = torch.from_numpy(X).cuda().to(torch.bfloat16)
    loss, gW, gb = mlp.loss_and_grads(Xb, torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda(),
                                      torch.from_numpy(tgt).cuda())
    W = [w.cpu().numpy().astype(np.float64) for w in mlp.W]
    b = [v.cpu().numpy().astype(np.float64) for v in mlp.b]
    rloss, rgW, rgb = omlp.loss_and_grads(Xb.float().cpu().numpy(), W, b, lo, hi, tgt)
    assert _rel(loss.cpu().numpy(), rloss) < 2e-2
    for i in range(4):
        assert _rel(gW[i].cpu().numpy(), rgW[i]) < 2e-2, i
        assert _rel(gb[i].cpu().numpy(), rgb[i]) < 2e-2, i


def test_training_reduces_loss(engine):
    torch = pytest.importorskip("torch")
    from piquasso_gb300 import proposal

    rng = np.random.default_rng(1)
    M = 4096
    X = rng.normal(size=(M, proposal.F)).astype(np.float32)
    tgt = (X[:, 1] > 0).astype(np.int8) + 2 * (X[:, 2] > 0.5).astype(np.int8)  # learnable rule
    lo = np.zeros(M, dtype=np.int8)
    hi = np.full(M, 4, dtype=np.int8)
    mlp = proposal.MLP(seed=0)
    Xb = torch.from_numpy(X).cuda().to(torch.bfloat16)
    lo_t, hi_t, tg_t = (torch.from_numpy(a).cuda() for a in (lo, hi, tgt))
    first = None
    for _ in range(60):
        loss, gW, gb = mlp.loss_and_grads(Xb, lo_t, hi_t, tg_t)
        if first is None:
            first = float(loss.mean())
        mlp.adam(gW, gb, lr=3e-3)
    last = float(mlp.loss_and_grads(Xb, lo_t, hi_t, tg_t)[0].mean())
    assert last < 0.3 * first, (first, last)


def test_device_proposal_matches_training_path(engine):
    """log q(y) accumulated by the device sampler equals the log-likelihood of
    the same patterns through features() + forward + masked softmax."""
    torch = pytest.importorskip("torch")
    from piquasso_gb300 import metropolis, proposal

    d, n = 12, 6
    U = haar_unitary(d, 9)
    inp = np.array([1] * n + [0] * (d - n))
    stats = proposal.ModeStats(U, inp)
    mlp = proposal.MLP(seed=5)
    ps = metropolis.ProposalSampler(mlp, stats, 256)
    y, lq = ps.propose(seed=77)
    Y = y.cpu().numpy().astype(np.int64)
    assert np.all(Y.sum(axis=1) == n) and Y.max() <= proposal.CAP
    X, lo, hi, tgt = proposal.features(stats, Y)
    Xb = torch.from_numpy(X.reshape(-1, proposal.F)).cuda().to(torch.bfloat16)
    loss, _, _ = mlp.loss_and_grads(Xb, torch.from_numpy(lo.reshape(-1)).cuda(),
                                    torch.from_numpy(hi.reshape(-1)).cuda(), torch.from_numpy(tgt.reshape(-1)).cuda())
    nll = loss.cpu().numpy().reshape(len(Y), d).sum(axis=1)
    assert np.allclose(-nll, lq.cpu().numpy(), atol=1e-3), np.max(np.abs(-nll - lq.cpu().numpy()))


@pytest.mark.parametrize("B,d,n", [(256, 12, 6), (1000, 48, 24), (130, 20, 11)])
def test_fused_proposal_step_matches_separate_kernels(engine, B, d, n):
    """The fused tensor-core step (features, four layers on tcgen05, draw in
    one kernel per mode) draws the same patterns and log q, bit for bit, as
    the separate feature, GEMM and sampling kernels; batches that are not a
    multiple of the 128-chain tile included."""
    pytest.importorskip("torch")
    from piquasso_gb300 import metropolis, proposal

    U = haar_unitary(d, 3)
    inp = np.array([1] * n + [0] * (d - n))
    stats = proposal.ModeStats(U, inp)
    mlp = proposal.MLP(seed=11)
    fused = metropolis.ProposalSampler(mlp, stats, B, fused=True)
    sep = metropolis.ProposalSampler(mlp, stats, B, fused=False)
    for seed in (5, 2**63 + 7):
        yf, lqf = fused.propose(seed=seed)
        yf, lqf = yf.cpu().numpy().copy(), lqf.cpu().numpy().copy()
        ys, lqs = sep.propose(seed=seed)
        assert np.array_equal(yf, ys.cpu().numpy())
        assert np.array_equal(lqf, lqs.cpu().numpy())
        assert np.all(yf.astype(np.int64).sum(axis=1) == n)
    L = __import__("piquasso_gb300._lib", fromlist=["load"]).load()
    import ctypes

    code = ctypes.c_int32(-1)
    assert L.pqg_mlp_tc_status(ctypes.byref(code)) == 0 and code.value == 0


def test_metropolis_small_matches_exact_marginals(engine):
    """n=4 photons in d=8 modes: every pattern is reachable (occupations <= 4),
    so the chain targets the exact distribution; its two-mode marginals agree
    with the binomial-moment marginals."""
    from piquasso_gb300 import marginals, metropolis

    d, n = 8, 4
    U = haar_unitary(d, 12)
    inp = np.array([1] * n + [0] * (d - n))
    out = metropolis.run_chains(U, inp, mlp=None, chains=512, steps=120, burn_in=20, seed=3, baseline=True)
    S = out["samples"]
    assert 0.05 < out["acceptance"] <= 1.0
    tv = marginals.tvd_two_mode(S, inp, U, [(0, 1), (2, 5), (6, 7)])
    assert np.all(tv < 0.02), tv


def test_trained_network_gains_over_the_sampler_without_it(engine):
    """n = 14 photons in d = 28 modes (inside the training range n = 12..16),
    on a Haar(28) interferometer held out of training (seed 14500; training
    used seeds 1000 n + u, u < 13).  The same independence Metropolis sampler,
    equal chains and steps, with the shipped network as its proposal and
    without it (each mode's exact one-mode marginal, drawn in turn): with the
    network the acceptance is higher, the chains decorrelate faster (smaller
    integrated autocorrelation time of the mode occupations), and the two-mode
    marginals are within TVD 0.01 of the exact ones."""
    from piquasso_gb300 import metropolis, proposal

    n, d = 14, 28
    U = haar_unitary(d, 14500)
    inp = np.array([1] * n + [0] * (d - n))
    kw = dict(chains=1024, steps=400, burn_in=30, seed=5, pair_seed=1, n_pairs=16)
    learned = metropolis.evaluate(U, inp, mlp=proposal.load_mlp(), **kw)
    plain = metropolis.evaluate(U, inp, baseline=True, **kw)
    assert learned["acceptance"] > plain["acceptance"], (learned["acceptance"], plain["acceptance"])
    assert learned["tau_max"] < plain["tau_max"], (learned["tau_max"], plain["tau_max"])
    assert learned["tvd_max"] <= 0.01, learned["tvd_max"]
