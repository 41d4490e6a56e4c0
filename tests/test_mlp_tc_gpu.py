"""GPU: the tcgen05 GEMM of the MLP (pqg_mlp_gemm_tc) against a plain PyTorch
FP32 matmul of the same BF16 operands, over ragged shapes (M, N, K not
multiples of the 128 x BN x 64 tiles, N below 16, K below 16), every
epilogue, split-K, and the transpose kernel.  After each call the kernel's
device error code (a bounded wait that ran out) must be 0.

Tolerance: |C - ref| <= 1e-5 * (|A| |B|^T) + 1e-6 per entry (FP32 sums of the
same exact BF16 products in a different order); GELU epilogues are checked
against torch's exact (erf) GELU at 1e-5 relative plus the BF16 rounding of
the stored activation.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(300, 256, 256), (128, 256, 16), (1000, 8, 256), (77, 200, 104), (20, 16, 8), (513, 24, 136),
          (4096, 256, 256), (256, 256, 4096)]


def _f(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float)) if t is not None else None


def _v(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _status(L):
    code = np.zeros(1, dtype=np.int32)
    assert L.pqg_mlp_tc_status(code.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) == 0
    return int(code[0])


def _operands(torch, M, N, K, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    ref = A.float() @ B.float().t()
    scale = A.float().abs() @ B.float().abs().t()
    return A, B, ref, scale


@pytest.fixture(scope="module")
def L(engine):
    import torch

    torch.backends.cuda.matmul.allow_tf32 = False
    from piquasso_gb300 import _lib

    return _lib.load()


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_plain_and_bias(L, M, N, K):
    import torch

    A, B, ref, scale = _operands(torch, M, N, K, M + N + K)
    C = torch.empty(M, N, device="cuda")
    assert L.pqg_mlp_gemm_tc(_v(A), K, _v(B), K, M, N, K, 0, _f(C), None, None, None, None, 0, None) == 0
    torch.cuda.synchronize()
    assert _status(L) == 0
    assert torch.all((C - ref).abs() <= 1e-5 * scale + 1e-6)
    bias = torch.randn(N, device="cuda")
    assert L.pqg_mlp_gemm_tc(_v(A), K, _v(B), K, M, N, K, 3, _f(C), None, _f(bias), None, None, 0, None) == 0
    torch.cuda.synchronize()
    assert _status(L) == 0
    assert torch.all((C - ref - bias).abs() <= 1e-5 * scale + 1e-6)


@pytest.mark.parametrize("M,N,K", SHAPES[:5])
def test_gelu_epilogues(L, M, N, K):
    import torch

    A, B, ref, scale = _operands(torch, M, N, K, 7 * M + K)
    bias = torch.randn(N, device="cuda")
    pre = torch.empty(M, N, device="cuda")
    act = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    assert L.pqg_mlp_gemm_tc(_v(A), K, _v(B), K, M, N, K, 1, _f(pre), _v(act), _f(bias), None, None, 0, None) == 0
    torch.cuda.synchronize()
    assert _status(L) == 0
    want = ref + bias
    assert torch.all((pre - want).abs() <= 1e-5 * scale + 1e-6)
    g = torch.nn.functional.gelu(pre)
    assert torch.all((act.float() - g).abs() <= 2.0 ** -8 * g.abs() + 1e-5)
    # backward through the activation: C = acc * GELU'(p)
    p = torch.randn(M, N, device="cuda")
    d = torch.empty(M, N, device="cuda")
    db = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    assert L.pqg_mlp_gemm_tc(_v(A), K, _v(B), K, M, N, K, 4, _f(d), _v(db), None, _f(p), None, 0, None) == 0
    torch.cuda.synchronize()
    assert _status(L) == 0
    pr = p.clone().requires_grad_(True)
    torch.nn.functional.gelu(pr).sum().backward()
    gg = pr.grad
    assert torch.all((d - ref * gg).abs() <= 1e-5 * scale * gg.abs() + 1e-5 * (ref * gg).abs() + 1e-6)
    assert torch.all((db.float() - d).abs() <= 2.0 ** -8 * d.abs() + 1e-30)


@pytest.mark.parametrize("splits", [1, 3, 16, 40])
@pytest.mark.parametrize("M,N", [(256, 136), (255, 135)])
def test_split_k(L, splits, M, N):
    """K not a multiple of the 64-wide chunk; M N a multiple of 4 takes the
    float4 reduction (16 split lanes), 255 x 135 the one-thread-per-output
    one."""
    import torch

    K = 3000
    A, B, ref, scale = _operands(torch, M, N, K, splits)
    A2 = torch.zeros(M, 3008, device="cuda", dtype=torch.bfloat16)  # row stride 3008 (16-byte rows)
    A2[:, :K] = A
    B2 = torch.zeros(N, 3008, device="cuda", dtype=torch.bfloat16)
    B2[:, :K] = B
    C = torch.empty(M, N, device="cuda")
    scratch = torch.empty(splits * M * N, device="cuda")
    assert L.pqg_mlp_gemm_tc(_v(A2), 3008, _v(B2), 3008, M, N, K, 2, _f(C), None, None, None, _f(scratch), splits,
                             None) == 0
    torch.cuda.synchronize()
    assert _status(L) == 0
    assert torch.all((C - ref).abs() <= 1e-5 * scale + 1e-6)


@pytest.mark.parametrize("K", [12, 20, 3])
def test_k_not_a_multiple_of_8_ignores_the_row_padding(L, K):
    """K below the row stride (16-byte rows) with NaN in the padding: the TMA
    loads must fill the chunk past K with zeros, not read the padding."""
    import torch

    M, N = 300, 64
    A, B, ref, scale = _operands(torch, M, N, K, K)
    ld = (K + 7) // 8 * 8 + 8
    A2 = torch.full((M, ld), float("nan"), device="cuda").to(torch.bfloat16)
    B2 = torch.full((N, ld), float("nan"), device="cuda").to(torch.bfloat16)
    A2[:, :K] = A
    B2[:, :K] = B
    C = torch.empty(M, N, device="cuda")
    assert L.pqg_mlp_gemm_tc(_v(A2), ld, _v(B2), ld, M, N, K, 0, _f(C), None, None, None, None, 0, None) == 0
    torch.cuda.synchronize()
    assert _status(L) == 0
    assert torch.all((C - ref).abs() <= 1e-5 * scale + 1e-6)


def test_transpose_and_rejects(L):
    import torch

    X = torch.randn(77, 40, device="cuda").to(torch.bfloat16)
    Y = torch.zeros(40, 80, device="cuda", dtype=torch.bfloat16)
    assert L.pqg_mlp_transpose_bf16(_v(X), 77, 40, 40, _v(Y), 80, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(Y[:, :77], X.t())
    C = torch.empty(4, 4, device="cuda")
    # row strides that are not multiples of 8 elements are refused on the host
    assert L.pqg_mlp_gemm_tc(_v(X), 12, _v(X), 12, 4, 4, 12, 0, _f(C), None, None, None, None, 0, None) != 0


@pytest.mark.parametrize("rows,cols,ld_src,ld_dst", [(65536, 256, 256, 65536), (192, 128, 136, 200),
                                                     (128, 64, 64, 130), (64, 96, 96, 64)])
def test_transpose_tiles(L, rows, cols, ld_src, ld_dst):
    """Whole 64 x 64 tiles with 16-byte aligned rows take the tiled kernel
    (16-byte loads, 32-byte stores); ld_dst = 130 and cols = 96 fall back to
    the 32 x 32 kernel.  Either way the bits of src^T, and nothing written
    outside it."""
    import torch

    X = torch.randn(rows, ld_src, device="cuda").to(torch.bfloat16)
    Y = torch.full((cols, ld_dst), 7.0, device="cuda", dtype=torch.bfloat16)
    assert L.pqg_mlp_transpose_bf16(_v(X), rows, cols, ld_src, _v(Y), ld_dst, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(Y[:, :rows], X[:, :cols].t())
    assert torch.all(Y[:, rows:] == 7.0)


@pytest.mark.parametrize("M,N", [(65536, 256), (300, 8), (1, 40)])
def test_bias_grad(L, M, N):
    import torch

    d = torch.randn(M, N, device="cuda")
    db = torch.empty(N, device="cuda")
    part = torch.empty(((M + 255) // 256) * N, device="cuda")
    assert L.pqg_mlp_bias_grad(_f(d), M, N, _f(db), _f(part), None) == 0
    torch.cuda.synchronize()
    ref = d.double().sum(dim=0)
    assert torch.all((db.double() - ref).abs() <= 1e-5 * d.abs().double().sum(dim=0) + 1e-6)
    db2 = torch.empty(N, device="cuda")
    assert L.pqg_mlp_bias_grad(_f(d), M, N, _f(db2), _f(part), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(db, db2)  # deterministic


@pytest.mark.parametrize("M,N,K", [(65536, 256, 256), (40000, 256, 16), (50001, 48, 200), (39000, 8, 256)])
@pytest.mark.parametrize("epi", [0, 1, 3, 4])
def test_persistent_kernel_is_bitwise_the_tile_kernel(L, M, N, K, epi):
    """From 2 x SMs row tiles on (K <= 256, N <= 256, no split-K) the GEMM runs
    as the persistent kernel (B resident in shared memory, two TMEM
    accumulators).  The same rows computed as blocks of 16384 (below that
    threshold: one tile per CTA) must give the same bits, in every output of
    the epilogue; and the result against the FP32 reference as above."""
    import torch

    A, B, ref, scale = _operands(torch, M, N, K, M + 3 * epi)
    bias = torch.randn(N, device="cuda")
    pre = torch.randn(M, N, device="cuda")
    outs = []
    for blocks in (False, True):
        C = torch.full((M, N), float("nan"), device="cuda")
        Cb = torch.zeros(M, N, device="cuda", dtype=torch.bfloat16)
        step = 16384 if blocks else M
        for r0 in range(0, M, step):
            m = min(step, M - r0)
            a = A[r0:r0 + m]
            assert L.pqg_mlp_gemm_tc(_v(a), K, _v(B), K, m, N, K, epi, _f(C[r0:r0 + m]),
                                     _v(Cb[r0:r0 + m]) if epi in (1, 4) else None, _f(bias) if epi in (1, 3) else None,
                                     _f(pre[r0:r0 + m]) if epi == 4 else None, None, 0, None) == 0
        torch.cuda.synchronize()
        assert _status(L) == 0
        outs.append((C, Cb))
    assert torch.equal(outs[0][0], outs[1][0])
    assert torch.equal(outs[0][1], outs[1][1])
    if epi == 0:
        assert torch.all((outs[0][0] - ref).abs() <= 1e-5 * scale + 1e-6)


def test_adam_multi_matches_per_tensor(L):
    """pqg_mlp_adam_multi: every tensor's step in one launch, with the BF16
    copy and the transposed BF16 copy, equal bit for bit to pqg_mlp_adam per
    tensor (and the transposed copy to the copy's transpose); tensors without
    copies (biases) and a NULL copy array."""
    import torch

    gen = torch.Generator(device="cuda").manual_seed(3)
    shapes = [(256, 256), (16, 256), (256, 8), (1, 256), (3, 5)]
    base = []
    for r, c in shapes:
        base.append([torch.randn(r, c, device="cuda", generator=gen), torch.randn(r, c, device="cuda", generator=gen),
                     0.1 * torch.randn(r, c, device="cuda", generator=gen),
                     torch.rand(r, c, device="cuda", generator=gen)])
    lr, b1, b2, eps, step = 1e-3, 0.9, 0.999, 1e-8, 3
    one = [[t.clone() for t in x] for x in base]
    wb1 = [torch.empty(r, c, device="cuda", dtype=torch.bfloat16) for r, c in shapes]
    for i, (w, g, m1, m2) in enumerate(one):
        assert L.pqg_mlp_adam(_f(w), _v(wb1[i]) if i < 3 else None, _f(g), _f(m1), _f(m2), w.numel(), lr, b1, b2,
                              eps, step, None) == 0
    multi = [[t.clone() for t in x] for x in base]
    wb2 = [torch.empty(r, c, device="cuda", dtype=torch.bfloat16) for r, c in shapes]
    wbt2 = [torch.empty(c, r, device="cuda", dtype=torch.bfloat16) for r, c in shapes]
    n = len(shapes)
    P = ctypes.c_void_p * n
    R = ctypes.c_int64 * n
    arrs = [P(*[x[k].data_ptr() for x in multi]) for k in range(4)]
    wb_arr = P(*[wb2[i].data_ptr() if i < 3 else None for i in range(n)])
    wbt_arr = P(*[wbt2[i].data_ptr() if i < 3 else None for i in range(n)])
    rows, cols = R(*[r for r, _ in shapes]), R(*[c for _, c in shapes])
    assert L.pqg_mlp_adam_multi(n, arrs[0], wb_arr, wbt_arr, arrs[1], arrs[2], arrs[3], rows, cols, lr, b1, b2, eps,
                                step, None) == 0
    torch.cuda.synchronize()
    for i in range(n):
        for k in (0, 2, 3):  # weights and both moments
            assert torch.equal(one[i][k], multi[i][k]), (i, k)
        if i < 3:
            assert torch.equal(wb1[i], wb2[i])
            assert torch.equal(wbt2[i], wb2[i].t())
    # no copy arrays at all: the FP32 step alone
    again = [[t.clone() for t in x] for x in base]
    arrs = [P(*[x[k].data_ptr() for x in again]) for k in range(4)]
    assert L.pqg_mlp_adam_multi(n, arrs[0], None, None, arrs[1], arrs[2], arrs[3], rows, cols, lr, b1, b2, eps,
                                step, None) == 0
    torch.cuda.synchronize()
    assert all(torch.equal(one[i][0], again[i][0]) for i in range(n))
    assert L.pqg_mlp_adam_multi(17, arrs[0], None, None, arrs[1], arrs[2], arrs[3], rows, cols, lr, b1, b2, eps,
                                step, None) != 0


@pytest.mark.parametrize("M,N,K", [(65536, 256, 256), (50008, 48, 200), (50001, 48, 200), (1000, 256, 256),
                                   (40000, 40, 64)])
@pytest.mark.parametrize("epi", [1, 4])
def test_gemm_with_transposed_output(L, M, N, K, epi):
    """pqg_mlp_gemm_tc_t: the same C and BF16 output as pqg_mlp_gemm_tc, bit
    for bit, plus that BF16 output transposed (N x ld_t, ld_t >= M) and the
    column sums of C (deterministic, against a float64 sum).  The
    persistent kernel writes it from its epilogue at M a multiple of 8 (65536
    rows, and 50008 with a last tile of 88 rows); 50001 rows, 1000 rows (the
    one-tile kernel) and N = 40 (the register-store form) run the transpose
    after the GEMM.  Columns of the transposed output past M stay untouched."""
    import torch

    A, B, ref, scale = _operands(torch, M, N, K, M + N + epi)
    bias = torch.randn(N, device="cuda")
    pre = torch.randn(M, N, device="cuda")
    ld_t = (M + 7) // 8 * 8 + 8
    outs = []
    for with_t in (False, True):
        # 40 sentinel rows after each output: the row dimension is clipped exactly
        C_all = torch.full((M + 40, N), float("nan"), device="cuda")
        Cb_all = torch.full((M + 40, N), 5.0, device="cuda", dtype=torch.bfloat16)
        C, Cb = C_all[:M], Cb_all[:M]
        CbT = torch.full((N, ld_t), 3.0, device="cuda", dtype=torch.bfloat16)
        args = (_v(A), K, _v(B), K, M, N, K, epi, _f(C), _v(Cb), _f(bias) if epi == 1 else None,
                _f(pre) if epi == 4 else None)
        if with_t:
            sums = torch.empty(N, device="cuda")
            scratch = torch.empty(4 * ((M + 127) // 128) * N, device="cuda")
            assert L.pqg_mlp_gemm_tc_t(*args, _v(CbT), ld_t, _f(sums), _f(scratch), None) == 0
        else:
            assert L.pqg_mlp_gemm_tc(*args, None, 0, None) == 0
        torch.cuda.synchronize()
        assert _status(L) == 0
        assert torch.all(torch.isnan(C_all[M:])) and torch.all(Cb_all[M:] == 5.0)
        outs.append((C, Cb, CbT))
    # the column sums of C (FP32 sums in a fixed order), and the same bits again
    want = outs[1][0].double().sum(dim=0)
    assert torch.all((sums.double() - want).abs() <= 1e-5 * outs[1][0].abs().double().sum(dim=0) + 1e-6)
    sums2 = torch.empty(N, device="cuda")
    assert L.pqg_mlp_gemm_tc_t(*args, _v(CbT), ld_t, _f(sums2), _f(scratch), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(sums, sums2)
    assert torch.equal(outs[0][0], outs[1][0])
    assert torch.equal(outs[0][1], outs[1][1])
    assert torch.equal(outs[1][2][:, :M], outs[1][1].t())
    assert torch.all(outs[1][2][:, M:] == 3.0)
    # only the BF16 epilogues, and a transposed row stride of at least M in multiples of 8
    C = torch.empty(M, N, device="cuda")
    assert L.pqg_mlp_gemm_tc_t(_v(A), K, _v(B), K, M, N, K, 0, _f(C), None, None, None, _v(CbT), ld_t, None, None,
                               None) != 0
    assert L.pqg_mlp_gemm_tc_t(_v(A), K, _v(B), K, M, N, K, epi, _f(C), _v(Cb), _f(bias), _f(pre), _v(CbT), ld_t - 4,
                               None, None, None) != 0
    # column sums without a scratch
    assert L.pqg_mlp_gemm_tc_t(_v(A), K, _v(B), K, M, N, K, epi, _f(C), _v(Cb), _f(bias), _f(pre), _v(CbT), ld_t,
                               _f(sums2), None, None) != 0
