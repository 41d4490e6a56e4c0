// C ABI of the GB300 permanent engine (declared in include/pqperm_gb300.h).
//
// Host side of every call: plan on the host (plan.cpp), one H2D copy of the
// plan, then on one stream: zero the work-queue head, the persistent walk
// kernel, the level-1 and level-2 double-double reductions, one D2H copy of
// the results.  Device and pinned host buffers are cached per process and
// grow on demand.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pqperm_gb300.h"
#include "kernel_table.h"
#include "plan.hpp"
#include "reduce.cuh"

namespace pqg {

namespace {

thread_local std::string g_err;
thread_local double g_walk_ms = 0.0, g_dev_ms = 0.0, g_walk_steps = 0.0, g_walk_flops = 0.0;
thread_local double g_h2d = 0.0, g_d2h = 0.0;
std::atomic<uint64_t> g_launches{0};

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define PQG_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(PQG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(n + n / 2, 1 << 16);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
};

struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(n + n / 2, 1 << 16);
        cudaError_t e = cudaMallocHost(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
};

struct Context {
    std::mutex mu;
    bool ready = false;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, evs = nullptr;
    DevBuf plan, partials, chunk_out, out, counter;
    HostBuf h_plan, h_out;
    PlanConfig cfg;
    std::vector<int> occ_cache[4];  // blocks per SM, per kernel table, per column count

    int init() {
        if (ready) return PQG_OK;
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) return fail(PQG_ERR_NO_DEVICE, "no CUDA device visible");
        PQG_CUDA(cudaGetDevice(&device));
        PQG_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
        PQG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        PQG_CUDA(cudaEventCreate(&ev0));
        PQG_CUDA(cudaEventCreate(&ev1));
        PQG_CUDA(cudaEventCreate(&ev2));
        PQG_CUDA(cudaEventCreate(&evs));
        cfg.num_sms = num_sms;
        for (auto &v : occ_cache) v.assign(PQG_MAX_COLS + 1, -1);
        ready = true;
        return PQG_OK;
    }
};

Context &ctx() {
    static Context c;
    return c;
}

const KernelInfo *table_for(Form form, Precision prec, int *which) {
    if (form == Form::PLAIN) {
        *which = prec == Precision::C128 ? 0 : 1;
        return prec == Precision::C128 ? k_plain_c128 : k_plain_c64;
    }
    *which = prec == Precision::C128 ? 2 : 3;
    return prec == Precision::C128 ? k_laplace_c128 : k_laplace_c64;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Runs a finished plan; writes n_outputs complex values (2*T each) to host `out`
// and, if out_lo != nullptr, the low words (2 doubles per output).
template <typename T>
int run_plan(Context &C, Planner &pl, T *out, double *out_lo) {
    const int64_t n_probs = static_cast<int64_t>(pl.probs.size());
    if (n_probs == 0) return PQG_OK;
    // pack the plan: problems | item_begin | chunks | arena
    const size_t o_probs = 0;
    const size_t o_items = align256(o_probs + sizeof(PqgProblem) * n_probs);
    const size_t o_chunks = align256(o_items + sizeof(int64_t) * (n_probs + 1));
    const size_t o_arena = align256(o_chunks + sizeof(PqgChunk) * std::max<size_t>(1, pl.chunks.size()));
    const size_t total = align256(o_arena + pl.arena.size());
    PQG_CUDA(C.h_plan.ensure(total));
    PQG_CUDA(C.plan.ensure(total));
    unsigned char *h = static_cast<unsigned char *>(C.h_plan.p);
    std::memcpy(h + o_probs, pl.probs.data(), sizeof(PqgProblem) * n_probs);
    std::memcpy(h + o_items, pl.item_begin.data(), sizeof(int64_t) * (n_probs + 1));
    if (!pl.chunks.empty()) std::memcpy(h + o_chunks, pl.chunks.data(), sizeof(PqgChunk) * pl.chunks.size());
    if (!pl.arena.empty()) std::memcpy(h + o_arena, pl.arena.data(), pl.arena.size());
    unsigned char *d = static_cast<unsigned char *>(C.plan.p);

    const size_t n_parts = static_cast<size_t>(std::max<int64_t>(1, pl.total_parts));
    PQG_CUDA(C.partials.ensure(n_parts * 4 * sizeof(double)));
    PQG_CUDA(C.chunk_out.ensure(std::max<size_t>(1, pl.chunks.size()) * PQG_MAX_OUT * 4 * sizeof(double)));
    const size_t out_bytes = static_cast<size_t>(pl.total_outputs) * 2 * sizeof(T);
    const size_t lo_bytes = static_cast<size_t>(pl.total_outputs) * 2 * sizeof(double);
    PQG_CUDA(C.out.ensure(align256(out_bytes) + lo_bytes));
    PQG_CUDA(C.h_out.ensure(align256(out_bytes) + lo_bytes));
    PQG_CUDA(C.counter.ensure(256));

    cudaStream_t s = C.stream;
    PQG_CUDA(cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, s));

    WalkArgs A;
    A.probs = reinterpret_cast<const PqgProblem *>(d + o_probs);
    A.item_begin = reinterpret_cast<const int64_t *>(d + o_items);
    A.arena = d + o_arena;
    A.counter = static_cast<unsigned long long *>(C.counter.p);
    A.partials = static_cast<double *>(C.partials.p);
    A.total_items = pl.total_items;
    A.n_probs = static_cast<int32_t>(n_probs);
    A.pad = 0;

    g_walk_ms = 0.0;
    g_dev_ms = 0.0;
    g_walk_steps = pl.total_steps;
    g_walk_flops = pl.total_flops;
    g_h2d = static_cast<double>(total);
    g_d2h = static_cast<double>(align256(out_bytes) + lo_bytes);
    PQG_CUDA(cudaEventRecord(C.evs, s));
    if (pl.total_items > 0) {
        int which = 0;
        const KernelInfo *tab = table_for(pl.form(), pl.precision(), &which);
        const KernelInfo &k = tab[pl.max_nc];
        int &occ = C.occ_cache[which][pl.max_nc];
        if (occ < 0) {
            if (k.smem_bytes > 48 * 1024)
                PQG_CUDA(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              static_cast<int>(k.smem_bytes)));
            int b = 0;
            PQG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k.fn, PQG_WALK_THREADS, k.smem_bytes));
            occ = std::max(1, b);
        }
        const int64_t warps_per_block = PQG_WALK_THREADS / 32;
        int64_t blocks = static_cast<int64_t>(C.num_sms) * occ;
        blocks = std::min<int64_t>(blocks, (pl.total_items + warps_per_block - 1) / warps_per_block);
        PQG_CUDA(cudaMemsetAsync(C.counter.p, 0, sizeof(unsigned long long), s));
        void *args[] = {&A};
        PQG_CUDA(cudaEventRecord(C.ev0, s));
        PQG_CUDA(cudaLaunchKernel(k.fn, dim3(static_cast<unsigned>(blocks)), dim3(PQG_WALK_THREADS), args,
                                  k.smem_bytes, s));
        PQG_CUDA(cudaEventRecord(C.ev1, s));
        g_launches++;
        if (!pl.chunks.empty()) {
            reduce_chunks<<<static_cast<unsigned>(pl.chunks.size()), 256, 0, s>>>(
                reinterpret_cast<const PqgChunk *>(d + o_chunks), A.probs, A.partials,
                static_cast<double *>(C.chunk_out.p));
            PQG_CUDA(cudaGetLastError());
            g_launches++;
        }
    }
    unsigned char *dout = static_cast<unsigned char *>(C.out.p);
    double *dlo = reinterpret_cast<double *>(dout + align256(out_bytes));
    finish_problems<T><<<static_cast<unsigned>((n_probs + 3) / 4), 128, 0, s>>>(
        A.probs, static_cast<int>(n_probs), static_cast<const double *>(C.chunk_out.p), reinterpret_cast<T *>(dout),
        dlo);
    PQG_CUDA(cudaGetLastError());
    g_launches++;
    PQG_CUDA(cudaEventRecord(C.ev2, s));
    unsigned char *hout = static_cast<unsigned char *>(C.h_out.p);
    PQG_CUDA(cudaMemcpyAsync(hout, dout, align256(out_bytes) + lo_bytes, cudaMemcpyDeviceToHost, s));
    PQG_CUDA(cudaStreamSynchronize(s));
    if (pl.total_items > 0) {
        float ms = 0.0f;
        PQG_CUDA(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
        g_walk_ms = ms;
    }
    {
        float ms = 0.0f;
        PQG_CUDA(cudaEventElapsedTime(&ms, C.evs, C.ev2));
        g_dev_ms = ms;
    }
    std::memcpy(out, hout, out_bytes);
    if (out_lo) std::memcpy(out_lo, hout + align256(out_bytes), lo_bytes);
    return PQG_OK;
}

std::vector<double> widen(const float *m, int64_t n) {
    std::vector<double> v(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) v[i] = static_cast<double>(m[i]);
    return v;
}

template <typename T>
int plain_batch(const double *matrix, int64_t nr, int64_t nc, const int32_t *rows, const int32_t *cols, int64_t batch,
                Precision prec, T *out, double *out_lo) {
    if (batch < 0 || nr < 0 || nc < 0 || !out) return fail(PQG_ERR_INVALID, "invalid arguments");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    // inputs are validated before the device is touched
    Planner pl(prec, Form::PLAIN, C.cfg);
    for (int64_t b = 0; b < batch; ++b) {
        std::string err;
        int st = pl.add(matrix, nr, nc, rows ? rows + b * nr : nullptr, cols ? cols + b * nc : nullptr, err);
        if (st) return fail(st, batch > 1 ? "problem " + std::to_string(b) + ": " + err : err);
    }
    int st = C.init();
    if (st) return st;
    pl.set_config(C.cfg);
    pl.finish();
    return run_plan<T>(C, pl, out, out_lo);
}

// Laplace permanents of `batch` problems sharing one matrix; problem b writes
// 2*nc values at out + 2*nc*b (its count, 1 or nc, to n_out[b]).
template <typename T>
int laplace_batch(const double *matrix, int64_t nr, int64_t nc, const int32_t *rows, const int32_t *cols,
                  int64_t batch, Precision prec, T *out, int64_t *n_out) {
    if (nr < 0 || nc < 0 || batch < 0 || !out) return fail(PQG_ERR_INVALID, "invalid arguments");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    PlanConfig cfg = C.cfg;
    cfg.p_max = std::min<int64_t>(cfg.p_max, 512);
    Planner pl(prec, Form::LAPLACE, cfg);
    for (int64_t b = 0; b < batch; ++b) {
        std::string err;
        int st = pl.add(matrix, nr, nc, rows ? rows + b * nr : nullptr, cols ? cols + b * nc : nullptr, err);
        if (st) return fail(st, batch > 1 ? "problem " + std::to_string(b) + ": " + err : err);
    }
    int st = C.init();
    if (st) return st;
    cfg.num_sms = C.cfg.num_sms;
    pl.set_config(cfg);
    pl.finish();
    std::vector<T> res(2 * static_cast<size_t>(std::max<int64_t>(1, pl.total_outputs)));
    st = run_plan<T>(C, pl, res.data(), nullptr);
    if (st) return st;
    const int64_t stride = 2 * std::max<int64_t>(1, nc);
    for (int64_t b = 0; b < batch; ++b) {
        const PendingProblem &pp = pl.pending[static_cast<size_t>(b)];
        const int64_t oi = pl.probs[static_cast<size_t>(b)].out_index;
        T *o = out + b * stride;
        if (pp.kind == PQG_KIND_CONSTANT) {
            for (int64_t j = 0; j < stride; ++j) o[j] = T(0);
            o[0] = res[2 * oi];
            o[1] = res[2 * oi + 1];
            if (n_out) n_out[b] = 1;
            continue;
        }
        for (int64_t j = 0; j < nc; ++j) {
            const int slot = pp.out_map[static_cast<size_t>(j)];
            o[2 * j] = res[2 * (oi + slot)];
            o[2 * j + 1] = res[2 * (oi + slot) + 1];
        }
        if (n_out) n_out[b] = nc;
    }
    return PQG_OK;
}

template <typename T>
int laplace_one(const double *matrix, int64_t nr, int64_t nc, const int32_t *rows, const int32_t *cols,
                Precision prec, T *out, int64_t *n_out) {
    return laplace_batch<T>(matrix, nr, nc, rows, cols, 1, prec, out, n_out);
}

// ------------------------------------------------------------ peak probes
template <typename F, int CHAINS>
__global__ void fma_chains(F *out, int iters, F b, F c) {
    F a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = static_cast<F>(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = a[k] * b + c;
    }
    F s = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    if (s == static_cast<F>(-1.2345)) out[0] = s;  // keeps the chains live
}

template <typename F, int CHAINS>
int time_fma(Context &C, double target_ms, double *tflops) {
    const int threads = 256;
    int occ = 0;
    PQG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fma_chains<F, CHAINS>, threads, 0));
    const int blocks = C.num_sms * std::max(1, occ);
    PQG_CUDA(C.out.ensure(1024));
    F *o = static_cast<F *>(C.out.p);
    int iters = 256;
    for (int rep = 0; rep < 8; ++rep) {
        fma_chains<F, CHAINS><<<blocks, threads, 0, C.stream>>>(o, iters, static_cast<F>(0.999999), static_cast<F>(1e-7));
        PQG_CUDA(cudaEventRecord(C.ev0, C.stream));
        fma_chains<F, CHAINS><<<blocks, threads, 0, C.stream>>>(o, iters, static_cast<F>(0.999999), static_cast<F>(1e-7));
        PQG_CUDA(cudaEventRecord(C.ev1, C.stream));
        PQG_CUDA(cudaEventSynchronize(C.ev1));
        g_launches += 2;
        float ms = 0.0f;
        PQG_CUDA(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
        const double flops = 2.0 * CHAINS * static_cast<double>(iters) * threads * blocks;
        *tflops = flops / (ms * 1e-3) / 1e12;
        if (ms >= 0.5 * target_ms || iters > (1 << 28)) break;
        iters = static_cast<int>(std::min<double>(iters * std::max(2.0, target_ms / std::max(ms, 1e-3f)), 1 << 29));
    }
    return PQG_OK;
}

}  // namespace

}  // namespace pqg

using namespace pqg;

extern "C" {

const char *pqg_last_error(void) { return g_err.c_str(); }

const char *pqg_version(void) { return "pqperm_gb300 0.1.0 (sm_103a)"; }

uint64_t pqg_kernel_launches(void) { return g_launches.load(); }

int pqg_permanent_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows, const int32_t *cols,
                       int32_t mode, double *out, double *out_lo) {
    (void)mode;
    return plain_batch<double>(matrix, n_rows, n_cols, rows, cols, 1, Precision::C128, out, out_lo);
}

int pqg_permanent_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows, const int32_t *cols,
                      float *out) {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return plain_batch<float>(m.data(), n_rows, n_cols, rows, cols, 1, Precision::C64, out, nullptr);
}

int pqg_permanent_batch_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                             const int32_t *cols, int64_t batch, int32_t mode, double *out) {
    (void)mode;
    return plain_batch<double>(matrix, n_rows, n_cols, rows, cols, batch, Precision::C128, out, nullptr);
}

int pqg_permanent_batch_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                            const int32_t *cols, int64_t batch, float *out) {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return plain_batch<float>(m.data(), n_rows, n_cols, rows, cols, batch, Precision::C64, out, nullptr);
}

int pqg_permanent_laplace_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                               const int32_t *cols, double *out, int64_t *n_out) {
    return laplace_one<double>(matrix, n_rows, n_cols, rows, cols, Precision::C128, out, n_out);
}

int pqg_permanent_laplace_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                              const int32_t *cols, float *out, int64_t *n_out) {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return laplace_one<float>(m.data(), n_rows, n_cols, rows, cols, Precision::C64, out, n_out);
}

int pqg_permanent_laplace_batch_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                                     const int32_t *cols, int64_t batch, double *out, int64_t *n_out) {
    return laplace_batch<double>(matrix, n_rows, n_cols, rows, cols, batch, Precision::C128, out, n_out);
}

int pqg_permanent_laplace_batch_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                                    const int32_t *cols, int64_t batch, float *out, int64_t *n_out) {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return laplace_batch<float>(m.data(), n_rows, n_cols, rows, cols, batch, Precision::C64, out, n_out);
}

int pqg_measure_vector_peaks(double ms, double *out2) {
    if (!out2) return fail(PQG_ERR_INVALID, "null output");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    int st = C.init();
    if (st) return st;
    st = time_fma<double, 8>(C, ms, &out2[0]);
    if (st) return st;
    return time_fma<float, 16>(C, ms, &out2[1]);
}

int pqg_last_timing(double *walk_ms, double *device_ms, double *steps, double *flops, double *h2d_bytes,
                    double *d2h_bytes) {
    if (h2d_bytes) *h2d_bytes = g_h2d;
    if (d2h_bytes) *d2h_bytes = g_d2h;
    if (walk_ms) *walk_ms = g_walk_ms;
    if (device_ms) *device_ms = g_dev_ms;
    if (steps) *steps = g_walk_steps;
    if (flops) *flops = g_walk_flops;
    return PQG_OK;
}

}  // extern "C"
