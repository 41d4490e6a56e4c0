"""Learned proposal for Metropolis boson sampling: an autoregressive MLP over
output occupations.

The model walks the output modes j = 0..d-1 in order and predicts the
occupation s_j in {0, ..., 7} from a fixed-size feature vector of mode j and
of the occupations already chosen, so one network serves any (n, d).  It is
trained by maximum likelihood on exact samples, and its log-probability
log q(s) = sum_j log softmax_j(s_j) is exact (every step is a normalised,
masked softmax), as an independence Metropolis proposal requires.

Per-mode inputs, computed once per interferometer from the exact one- and
two-mode statistics of the output (binomial moments, see marginals.py):
  * p_j(k): the exact one-mode marginal Pr(X_j = k), k = 0..4, and the
    tail Pr(X_j >= 5);
  * mu_j = E[X_j], var_j = Var[X_j];
  * C_kj = Cov(X_k, X_j) = |T_kj|^2 - 2 Q_kj for single-photon inputs, with
    T_kj = sum_a U_ka conj(U_ja) and Q_kj = sum_a |U_ka|^2 |U_ja|^2 over the
    occupied input modes a (the z_k z_j w_k w_j coefficient of the generating
    function of marginals.py).
Per-step state: photons left, modes left, and the linear-regression shift of
mode j's mean given the chosen occupations, sum_{k<j} C_kj (s_k - mu_k)/var_k.

Network: F = 16 features -> 256 -> 256 -> 256 -> 8 logits (GELU, BF16
weights and activations, FP32 accumulation and master weights), one per
occupation 0..7; classes that cannot complete a pattern (more photons than are
left, or too few to fill the remaining modes with at most 7 each) are masked.
Occupations above 7 have no support: at n=24, d=48 their exact probability is
about 1e-5 per mode, so the chain's target differs from the exact distribution
by well under the sampling noise.  (A softmax over 0..4 alone would leave about
13 % of the exact mass at n=24, d=48 unreachable.)  The GEMMs, GELU backward, masked softmax cross-entropy and
Adam run as this package's CUDA kernels (pqg_mlp_* in the C ABI); PyTorch
only holds the device buffers.
"""

import ctypes

import numpy as np

from . import _lib
from .marginals import marginals

F = 16          # features per (sample, mode)
HIDDEN = 256
CLASSES = 8     # occupations 0..7
LD = 8          # logit width
CAP = 7


class ModeStats:
    """Per-interferometer statistics feeding the features (single-photon inputs
    or general inputs for p_j and mu_j; C uses the single-photon formula)."""

    def __init__(self, U, input_photons):
        U = np.asarray(U, dtype=np.complex128)
        inp = np.asarray(input_photons, dtype=int)
        self.d = len(inp)
        self.n = int(inp.sum())
        act = np.nonzero(inp)[0]
        W = U[:, act]                        # U[output j, input a]
        P = np.abs(W) ** 2 * inp[act][None, :]
        self.mu = P.sum(axis=1)              # E[X_j]
        self.p = np.zeros((self.d, 5))
        self.tail = np.zeros(self.d)
        self.var = np.zeros(self.d)
        one_mode = marginals(inp, U, [(j,) for j in range(self.d)])  # one GPU call for every mode
        for j in range(self.d):
            m = one_mode[j]
            self.p[j] = m[:5]
            self.tail[j] = max(0.0, 1.0 - float(m[:5].sum()))
            k = np.arange(len(m))
            self.var[j] = float((m * k * k).sum() - (m * k).sum() ** 2)
        self.var = np.maximum(self.var, 1e-6)
        T = W @ W.conj().T                   # T_kj = sum_a U_ka conj(U_ja)
        Q = (np.abs(W) ** 2) @ (np.abs(W) ** 2).T
        self.C = np.abs(T) ** 2 - 2.0 * Q
        np.fill_diagonal(self.C, 0.0)
        self.mu_suffix = np.concatenate([np.cumsum(self.mu[::-1])[::-1], [0.0]])


def features(stats, samples):
    """Training features for every (sample, mode): array (S, d, F) float32,
    plus the class masks lo/hi (S, d) int8 and targets (S, d) int8."""
    S = np.asarray(samples, dtype=np.int64)
    ns, d = S.shape
    n = stats.n
    used = np.concatenate([np.zeros((ns, 1), dtype=np.int64), np.cumsum(S, axis=1)[:, :-1]], axis=1)
    n_rem = n - used                                     # photons left before mode j
    j = np.arange(d)[None, :]
    left = d - j                                         # modes left including j
    z = (S - stats.mu[None, :]) / stats.var[None, :]
    shift = z @ np.triu(stats.C, 1)                      # sum_{k<j} C_kj z_k
    X = np.zeros((ns, d, F), dtype=np.float32)
    X[..., 0] = 1.0
    X[..., 1] = n_rem / n
    X[..., 2] = left / d
    X[..., 3] = n_rem / left
    X[..., 4:9] = stats.p[None, :, :]
    X[..., 9] = stats.mu[None, :]
    X[..., 10] = (n_rem - stats.mu_suffix[None, :d]) / np.sqrt(n)
    X[..., 11] = shift
    X[..., 12] = stats.mu[None, :] + shift
    X[..., 13] = n_rem * stats.mu[None, :] / np.maximum(stats.mu_suffix[None, :d], 1e-12)
    X[..., 14] = stats.var[None, :]
    X[..., 15] = stats.tail[None, :]
    lo = np.maximum(0, n_rem - CAP * (left - 1)).astype(np.int8)
    hi = np.minimum(CAP, n_rem).astype(np.int8)
    return X, lo, hi, S.astype(np.int8)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class MLP:
    """Weights and the forward/backward passes on the engine's kernels.

    Every GEMM is C = A . B^T with both operands BF16 and K-major, on the
    tcgen05 kernel (pqg_mlp_gemm_tc): the forward pass reads the BF16 weights
    transposed (WbT[i], fan_out x fan_in), the data gradient reads them as
    stored (Wb[i]), and the weight gradient reads transposed copies of the
    activations and of the output gradient, which the GEMMs producing them
    write beside their outputs (pqg_mlp_gemm_tc_t; the features and the
    head's gradient go through pqg_mlp_transpose_bf16).  The data-gradient
    GEMMs also give the next layer's bias gradient (their output's column
    sums); Adam updates every tensor and the BF16 copies in one launch."""

    def __init__(self, seed=0, device="cuda"):
        import torch

        self.torch = torch
        g = torch.Generator().manual_seed(seed)
        dims = [(F, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, LD)]
        self.W, self.Wb, self.WbT, self.b, self.mW, self.vW, self.mb, self.vb = [], [], [], [], [], [], [], []
        for (fi, fo) in dims:
            w = torch.randn(fi, fo, generator=g) * (2.0 / fi) ** 0.5
            if fo == LD:
                w *= 0.1
            w = w.to(device)
            self.W.append(w)
            self.Wb.append(w.to(torch.bfloat16))
            self.WbT.append(w.t().contiguous().to(torch.bfloat16))
            self.b.append(torch.zeros(fo, device=device))
            self.mW.append(torch.zeros_like(w))
            self.vW.append(torch.zeros_like(w))
            self.mb.append(torch.zeros(fo, device=device))
            self.vb.append(torch.zeros(fo, device=device))
        self.step = 0
        self.device = device

    def state_dict(self):
        return {"W": [w.cpu().numpy() for w in self.W], "b": [b.cpu().numpy() for b in self.b], "step": self.step}

    def load_state_dict(self, sd):
        torch = self.torch
        for i in range(4):
            self.W[i] = torch.from_numpy(np.asarray(sd["W"][i], dtype=np.float32)).to(self.device)
            self.b[i] = torch.from_numpy(np.asarray(sd["b"][i], dtype=np.float32)).to(self.device)
            self._refresh_bf16(i)
        self.step = int(sd.get("step", 0))

    def _refresh_bf16(self, i):
        """BF16 copies of W[i]: as stored (Wb) and transposed (WbT)."""
        torch = self.torch
        self.Wb[i] = self.W[i].to(torch.bfloat16)
        fi, fo = self.W[i].shape
        self.WbT[i] = torch.empty(fo, fi, device=self.device, dtype=torch.bfloat16)
        self._transpose(self.Wb[i], self.WbT[i])

    # ---------------------------------------------------------------- kernels
    def _gemm(self, A, lda, B, ldb, M, N, K, epi, C, Cb=None, bias=None, pre=None, scratch=None, splits=0,
              stream=None):
        """C = A[M x K] . B[N x K]^T (BF16, K-major) with epilogue `epi`."""
        L = _lib.load()
        fp = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float)) if t is not None else None  # noqa
        st = L.pqg_mlp_gemm_tc(_ptr(A), lda, _ptr(B), ldb, M, N, K, epi, fp(C), _ptr(Cb) if Cb is not None else None,
                               fp(bias), fp(pre), fp(scratch), int(splits), stream)
        if st:
            raise RuntimeError("pqg_mlp_gemm_tc failed: " + _lib.last_error())

    def _gemm_t(self, A, lda, B, ldb, M, N, K, epi, C, Cb, bias=None, pre=None, col_sums=None, stream=None):
        """_gemm with a BF16 epilogue that also returns Cb^T (N x Mp, rows
        padded to a multiple of 8 elements), written by the GEMM itself, and
        fills `col_sums` (N floats, when given) with the column sums of C."""
        torch = self.torch
        L = _lib.load()
        Mp = (M + 7) // 8 * 8
        CbT = torch.empty(N, Mp, device=self.device, dtype=torch.bfloat16)
        scratch = None
        if col_sums is not None:
            scratch = torch.empty(4 * ((M + 127) // 128) * N, device=self.device, dtype=torch.float32)
        fp = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float)) if t is not None else None  # noqa
        st = L.pqg_mlp_gemm_tc_t(_ptr(A), lda, _ptr(B), ldb, M, N, K, epi, fp(C), _ptr(Cb), fp(bias), fp(pre),
                                 _ptr(CbT), Mp, fp(col_sums), fp(scratch), stream)
        if st:
            raise RuntimeError("pqg_mlp_gemm_tc_t failed: " + _lib.last_error())
        return CbT

    def _transpose(self, src, dst):
        """dst (cols x ld) = src (rows x cols)^T, BF16."""
        rows, cols = src.shape
        st = _lib.load().pqg_mlp_transpose_bf16(_ptr(src), rows, cols, src.stride(0), _ptr(dst), dst.stride(0), None)
        if st:
            raise RuntimeError("pqg_mlp_transpose_bf16 failed: " + _lib.last_error())

    def _transposed(self, src):
        """K-major copy of a (M x C) BF16 matrix for a GEMM over M: (C x Mp),
        rows padded to a multiple of 8 elements (16 bytes)."""
        M, C = src.shape
        Mp = (M + 7) // 8 * 8
        dst = self.torch.empty(C, Mp, device=self.device, dtype=self.torch.bfloat16)
        self._transpose(src, dst)
        return dst

    def forward(self, Xb, keep=False, stream=None):
        """Xb: (M, F) bf16 -> logits (M, LD) fp32 (+ activations if keep);
        `stream`: the CUDA stream of the GEMMs (None: the default stream)."""
        torch = self.torch
        M = Xb.shape[0]
        acts = [Xb]
        actsT = [None]
        pres = []
        h = Xb
        for i in range(3):
            pre = torch.empty(M, HIDDEN, device=self.device, dtype=torch.float32)
            act = torch.empty(M, HIDDEN, device=self.device, dtype=torch.bfloat16)
            fi = h.shape[1]
            if keep:  # the backward pass's weight gradient wants the activation transposed too
                actsT.append(self._gemm_t(h, fi, self.WbT[i], fi, M, HIDDEN, fi, 1, pre, act, bias=self.b[i],
                                          stream=stream))
            else:
                self._gemm(h, fi, self.WbT[i], fi, M, HIDDEN, fi, 1, pre, Cb=act, bias=self.b[i], stream=stream)
            pres.append(pre)
            acts.append(act)
            h = act
        logits = torch.empty(M, LD, device=self.device, dtype=torch.float32)
        self._gemm(h, HIDDEN, self.WbT[3], HIDDEN, M, LD, HIDDEN, 3, logits, bias=self.b[3], stream=stream)
        if keep:
            return logits, acts, actsT, pres
        return logits

    def loss_and_grads(self, Xb, lo, hi, target):
        """Mean masked cross-entropy (nats per mode) and weight gradients."""
        torch = self.torch
        L = _lib.load()
        M = Xb.shape[0]
        logits, acts, actsT, pres = self.forward(Xb, keep=True)
        loss = torch.empty(M, device=self.device, dtype=torch.float32)
        dz = torch.empty(M, LD, device=self.device, dtype=torch.float32)
        dzb = torch.empty(M, LD, device=self.device, dtype=torch.bfloat16)
        st = L.pqg_mlp_softmax_xent(ctypes.cast(logits.data_ptr(), ctypes.POINTER(ctypes.c_float)), M, LD, CLASSES,
                                    ctypes.cast(lo.data_ptr(), ctypes.POINTER(ctypes.c_int8)),
                                    ctypes.cast(hi.data_ptr(), ctypes.POINTER(ctypes.c_int8)),
                                    ctypes.cast(target.data_ptr(), ctypes.POINTER(ctypes.c_int8)), 1.0 / M,
                                    ctypes.cast(loss.data_ptr(), ctypes.POINTER(ctypes.c_float)),
                                    ctypes.cast(dz.data_ptr(), ctypes.POINTER(ctypes.c_float)), _ptr(dzb), None)
        if st:
            raise RuntimeError(_lib.last_error())
        grads_W, grads_b = [None] * 4, [None] * 4
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        d_out, d_out_b, d_out_t, d_out_sums = dz, dzb, None, None
        for i in (3, 2, 1, 0):
            fi, fo = self.W[i].shape
            # dW = h_in^T d_out: K = M (split over the batch), both operands K-major: the
            # transposed copies the GEMMs wrote (the features and the head's gradient: a transpose)
            hT = actsT[i] if actsT[i] is not None else self._transposed(acts[i])
            dT = d_out_t if d_out_t is not None else self._transposed(d_out_b)
            gW = torch.empty(fi, fo, device=self.device, dtype=torch.float32)
            # K splits of at least 512 rows, about one CTA per SM over the output tiles
            tiles = -(-fi // 128) * -(-fo // 256)
            splits = max(1, min(M // 512, sms // tiles))
            scratch = torch.empty(splits * fi * fo, device=self.device, dtype=torch.float32)
            self._gemm(hT, hT.shape[1], dT, dT.shape[1], fi, fo, M, 2, gW, scratch=scratch, splits=splits)
            if d_out_sums is not None:  # the column sums the data-gradient GEMM gave with d_out
                gb = d_out_sums
            else:
                gb = torch.empty(fo, device=self.device, dtype=torch.float32)
                part = torch.empty(((M + 255) // 256) * fo, device=self.device, dtype=torch.float32)
                st = L.pqg_mlp_bias_grad(ctypes.cast(d_out.data_ptr(), ctypes.POINTER(ctypes.c_float)), M, fo,
                                         ctypes.cast(gb.data_ptr(), ctypes.POINTER(ctypes.c_float)),
                                         ctypes.cast(part.data_ptr(), ctypes.POINTER(ctypes.c_float)), None)
                if st:
                    raise RuntimeError(_lib.last_error())
            grads_W[i], grads_b[i] = gW, gb
            if i == 0:
                break
            # d h_in = d_out W^T, through GELU'(pre) in the epilogue (FP32 and BF16)
            dh = torch.empty(M, fi, device=self.device, dtype=torch.float32)
            dhb = torch.empty(M, fi, device=self.device, dtype=torch.bfloat16)
            sums = torch.empty(fi, device=self.device, dtype=torch.float32)  # layer i - 1's bias gradient
            dht = self._gemm_t(d_out_b, fo, self.Wb[i], fo, M, fi, fo, 4, dh, dhb, pre=pres[i - 1], col_sums=sums)
            d_out, d_out_b, d_out_t, d_out_sums = dh, dhb, dht, sums
        return loss, grads_W, grads_b

    def adam(self, grads_W, grads_b, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        """One Adam step on every weight and bias, with the BF16 copies (Wb)
        and transposed copies (WbT) of the weights: one launch
        (pqg_mlp_adam_multi)."""
        L = _lib.load()
        self.step += 1
        ts = [(self.W[i], self.Wb[i], self.WbT[i], grads_W[i], self.mW[i], self.vW[i]) for i in range(4)]
        ts += [(self.b[i], None, None, grads_b[i], self.mb[i], self.vb[i]) for i in range(4)]
        P = ctypes.c_void_p * len(ts)
        arr = [P(*[(t[k].data_ptr() if t[k] is not None else None) for t in ts]) for k in range(6)]
        R = ctypes.c_int64 * len(ts)
        rows = R(*[t[0].shape[0] if t[0].dim() == 2 else 1 for t in ts])
        cols = R(*[t[0].shape[-1] for t in ts])
        st = L.pqg_mlp_adam_multi(len(ts), *arr, rows, cols, lr, b1, b2, eps, self.step, None)
        if st:
            raise RuntimeError(_lib.last_error())


DEFAULT_WEIGHTS = __import__("os").path.join(__import__("os").path.dirname(__file__), "data", "proposal_weights.npz")


def load_mlp(path=None, device="cuda"):
    """The trained network (default: the weights shipped with the package,
    produced by `python -m piquasso_gb300.train`)."""
    z = np.load(path or DEFAULT_WEIGHTS)
    mlp = MLP(seed=0, device=device)
    mlp.load_state_dict({"W": [z["W%d" % i] for i in range(4)], "b": [z["b%d" % i] for i in range(4)],
                         "step": int(z["step"]) if "step" in z else 0})
    return mlp
