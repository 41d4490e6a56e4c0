"""CPU oracle of the learned proposal's MLP — TEST INFRASTRUCTURE ONLY.

The network has no counterpart in the reference; this restates its forward
pass, masked softmax cross-entropy and backward pass in float64 numpy, with
BF16 rounding (round to nearest even) applied where the GPU kernels store or
stage BF16: the input features, the weights, every GEMM operand, and the GELU
activations.  Accumulation is float64 here and FP32 on the GPU, so gradients
agree to about 1e-3 relative.
"""

from math import erf, sqrt

import numpy as np

_erf = np.vectorize(erf)


def bf16(x):
    a = np.asarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / sqrt(2.0))) + x * np.exp(-0.5 * x * x) / sqrt(2.0 * np.pi)


def forward(X, W, b):
    """X (M, F); W[i] (fan_in, fan_out); b[i].  Returns logits, activations, pre-activations."""
    h = bf16(X)
    acts, pres = [h], []
    for i in range(3):
        pre = bf16(h) @ bf16(W[i]) + b[i]
        pres.append(pre)
        h = bf16(gelu(pre))
        acts.append(h)
    logits = bf16(h) @ bf16(W[3]) + b[3]
    return logits, acts, pres


def loss_and_grads(X, W, b, lo, hi, target, classes=5):
    M = X.shape[0]
    logits, acts, pres = forward(X, W, b)
    LD = logits.shape[1]
    dz = np.zeros_like(logits)
    loss = np.zeros(M)
    for m in range(M):
        cs = np.arange(lo[m], hi[m] + 1)
        z = logits[m, cs]
        mx = z.max()
        lse = mx + np.log(np.exp(z - mx).sum())
        loss[m] = lse - logits[m, target[m]]
        p = np.exp(logits[m, cs] - lse)
        dz[m, cs] = p
        dz[m, target[m]] -= 1.0
    dz /= M
    gW, gb = [None] * 4, [None] * 4
    d = dz
    for i in (3, 2, 1, 0):
        gW[i] = bf16(acts[i]).T @ bf16(d)
        gb[i] = d.sum(axis=0)
        if i == 0:
            break
        dh = bf16(d) @ bf16(W[i]).T
        d = dh * gelu_grad(pres[i - 1])
    assert LD >= classes
    return loss, gW, gb
