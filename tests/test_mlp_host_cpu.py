"""CPU tests of the learned proposal's training step on the host side: the
engine calls one step makes, and their arguments, recorded by a stand-in for
the engine library on CPU tensors (no GPU, nothing computed).

The step (proposal.py, MLP.loss_and_grads and MLP.adam) runs every GEMM on
the tcgen05 kernel: the hidden layers' forward GEMMs and the data-gradient
GEMMs through pqg_mlp_gemm_tc_t, which also writes their BF16 output
transposed (the weight gradient's K-major operand) and, for the data
gradients, the next layer's bias gradient; so a step transposes only the
features and the head's gradient, runs one separate bias gradient (the
head's), and one Adam launch for all eight tensors."""

import ctypes
from collections import Counter

import pytest

torch = pytest.importorskip("torch")

from piquasso_gb300 import _lib, proposal  # noqa: E402


class FakeEngine:
    """Records every call; every call succeeds."""

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        if not name.startswith("pqg_"):
            raise AttributeError(name)

        def call(*args):
            self.calls.append((name, args))
            return 0

        return call


@pytest.fixture()
def engine(monkeypatch):
    fake = FakeEngine()
    monkeypatch.setattr(_lib, "load", lambda: fake)

    class Props:
        multi_processor_count = 152

    monkeypatch.setattr(torch.cuda, "get_device_properties", lambda *a, **k: Props())
    return fake


def _addr(p):
    """The address a ctypes argument carries (None for NULL)."""
    if p is None:
        return None
    if isinstance(p, ctypes.c_void_p):
        return p.value
    return ctypes.cast(p, ctypes.c_void_p).value


def test_training_step_calls(engine):
    M = 4096
    mlp = proposal.MLP(seed=0, device="cpu")
    X = torch.zeros(M, proposal.F, dtype=torch.bfloat16)
    lo = torch.zeros(M, dtype=torch.int8)
    hi = torch.full((M,), proposal.CAP, dtype=torch.int8)
    tgt = torch.zeros(M, dtype=torch.int8)
    engine.calls.clear()
    loss, gW, gb = mlp.loss_and_grads(X, lo, hi, tgt)
    names = Counter(n for n, _ in engine.calls)
    assert names == Counter({"pqg_mlp_gemm_tc_t": 6, "pqg_mlp_gemm_tc": 5, "pqg_mlp_transpose_bf16": 2,
                             "pqg_mlp_bias_grad": 1, "pqg_mlp_softmax_xent": 1})
    gt = [a for n, a in engine.calls if n == "pqg_mlp_gemm_tc_t"]
    # forward: three bias + GELU GEMMs (epilogue 1) without column sums; backward:
    # three GELU' GEMMs (epilogue 4), each with the next layer's bias gradient
    assert [a[7] for a in gt] == [1, 1, 1, 4, 4, 4]
    assert all(a[14] is None and a[15] is None for a in gt[:3])
    assert all(a[14] is not None and a[15] is not None for a in gt[3:])
    # the transposed outputs: N x Mp with Mp = M rounded to 8 (row stride Mp)
    assert all(a[13] == M for a in gt)
    # the weight gradients (split-K, epilogue 2) read the transposed copies the
    # GEMMs wrote: A = the activation^T (row stride M), B = the gradient^T
    sk = [a for n, a in engine.calls if n == "pqg_mlp_gemm_tc" and a[7] == 2]
    assert len(sk) == 4
    t_out = [_addr(a[12]) for a in gt]
    # layers 3, 2, 1 read the activations of forward GEMMs 2, 1, 0; layers 2, 1, 0
    # the gradients of the backward GEMMs of layers 3, 2, 1
    assert [_addr(sk[k][0]) for k in range(3)] == [t_out[2], t_out[1], t_out[0]]
    assert [_addr(sk[k][2]) for k in (1, 2, 3)] == [t_out[3], t_out[4], t_out[5]]
    # splits: K = M rows over about one CTA per SM (152 SMs, 2 row tiles of 128 at fan-in 256)
    assert [a[13] for a in sk] == [min(M // 512, 152 // 2), min(M // 512, 152 // 2), min(M // 512, 152 // 2),
                                   min(M // 512, 152)]
    # the bias gradients: the head's from the softmax, the others are the column sums
    assert len(gb) == 4 and all(g is not None for g in gb)
    assert [tuple(g.shape) for g in gb] == [(proposal.HIDDEN,)] * 3 + [(proposal.LD,)]
    assert [_addr(gt[3 + k][14]) for k in range(3)] == [gb[2].data_ptr(), gb[1].data_ptr(), gb[0].data_ptr()]


def test_adam_one_launch(engine):
    mlp = proposal.MLP(seed=0, device="cpu")
    gW = [torch.zeros_like(w) for w in mlp.W]
    gb = [torch.zeros_like(b) for b in mlp.b]
    engine.calls.clear()
    mlp.adam(gW, gb, lr=2e-3)
    assert [n for n, _ in engine.calls] == ["pqg_mlp_adam_multi"]
    a = engine.calls[0][1]
    count, w, wb, wbt, g, m1, m2, rows, cols, lr, b1, b2, eps, step = a[:14]
    assert count == 8 and step == 1 and lr == 2e-3 and (b1, b2, eps) == (0.9, 0.999, 1e-8)
    assert list(w) == [t.data_ptr() for t in mlp.W + mlp.b]
    assert list(g) == [t.data_ptr() for t in gW + gb]
    assert list(m1) == [t.data_ptr() for t in mlp.mW + mlp.mb]
    assert list(m2) == [t.data_ptr() for t in mlp.vW + mlp.vb]
    # BF16 copies and transposed copies for the weights only
    assert list(wb) == [t.data_ptr() for t in mlp.Wb] + [None] * 4
    assert list(wbt) == [t.data_ptr() for t in mlp.WbT] + [None] * 4
    assert list(rows) == [w_.shape[0] for w_ in mlp.W] + [1] * 4
    assert list(cols) == [w_.shape[1] for w_ in mlp.W] + [b_.shape[0] for b_ in mlp.b]
    assert all(tuple(t.shape) == (c, r) for t, r, c in zip(mlp.WbT, list(rows), list(cols)))
    mlp.adam(gW, gb)
    assert engine.calls[-1][1][13] == 2  # the step count advances
