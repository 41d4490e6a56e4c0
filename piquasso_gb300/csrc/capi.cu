// C ABI of the GB300 permanent engine (declared in include/pqperm_gb300.h).
//
// Host side of every call: plan on the host (plan.cpp: problem descriptors,
// weight tables and the matrix, no per-problem matrix data), one H2D copy of
// the plan, then on one stream: the prep kernel that builds every problem's
// seeds, step rows and prefix tables from the matrix (prep.cuh), zero the
// work-queue head, the persistent walk kernel, the level-1 and level-2
// double-double reductions, one D2H copy of the results.  Device and pinned
// host buffers are cached per process and grow on demand.
#include <exception>
#include <new>
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pqperm_gb300.h"
#include "kernel_table.h"
#include "plan.hpp"
#include "prep.cuh"
#include "reduce.cuh"
#include "draw.cuh"

namespace pqg {

namespace {

thread_local std::string g_err;
thread_local double g_walk_ms = 0.0, g_dev_ms = 0.0, g_walk_steps = 0.0, g_walk_flops = 0.0;
thread_local double g_h2d = 0.0, g_d2h = 0.0;
// walk instantiation of the calling thread's last plan run: kernel table
// (PQG_WALK_* in the header) and exact column count; -1 / 0 when no walk ran
thread_local int g_last_table = -1, g_last_nc = 0;
std::atomic<uint64_t> g_launches{0};

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

// No C++ exception crosses the C ABI: every int entry point is a function-try-
// block whose handler turns the exception in flight (std::bad_alloc from
// the planner's host buffers, in practice) into PQG_ERR_HOST.
int host_failure() {
    try {
        throw;
    } catch (const std::bad_alloc &) {
        g_err = "out of host memory";
    } catch (const std::exception &e) {
        g_err = e.what();
    } catch (...) {
        g_err = "host-side failure";
    }
    return PQG_ERR_HOST;
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

// Device buffers of one executable plan.
struct DeviceBuffers {
    DevBuf plan, partials, chunk_out, out, counter, delta, draw;
};

// One autotuned setting: the planner knobs for the workloads of one form and
// arithmetic whose largest column count, total Gray-code steps and problem
// count fall in the given ranges (pqg_tuning_add).
struct TuneEntry {
    int32_t form, arith;        // 0 plain / 1 Laplace; 0 FP64, 1 double-float, 2 complex64
    int32_t nc_lo, nc_hi;       // largest column count, inclusive
    double steps_lo, steps_hi;  // total Gray-code steps, [lo, hi)
    int64_t probs_lo, probs_hi; // problems, inclusive
    int64_t items_per_smsp, p_max, seed_steps;
    int32_t blocks_per_sm;
};

// Locks: `mu` serialises the device work (buffers, stream, events) and is
// held by a launch until its results are back; `cfg_mu` guards the planner
// configuration and the tuning table, so that a thread planning its batch
// reads them without waiting for another thread's launch.  Writers of the
// configuration take mu, then cfg_mu (readers may hold either).
struct Context {
    std::mutex mu, cfg_mu;
    DeviceBuffers bufs;
    std::atomic<bool> ready{false};  // set once by init(), under mu
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, evs = nullptr;
    HostBuf h_plan, h_out;
    PlanConfig cfg;
    int blocks_per_sm = 0;  // process-wide walk blocks per SM (pqg_set_blocks_per_sm); 0: the plan's
    std::vector<TuneEntry> tune;  // autotuned settings by workload (pqg_tuning_add)
    std::vector<int> occ_cache[11];  // blocks per SM, per kernel table, per column count

    int init() {  // caller holds mu
        if (ready.load(std::memory_order_acquire)) return PQG_OK;
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
        {
            std::lock_guard<std::mutex> lock(cfg_mu);
            cfg.num_sms = num_sms;
        }
        for (auto &v : occ_cache) v.assign(PQG_MAX_COLS + 1, -1);
        ready.store(true, std::memory_order_release);
        return PQG_OK;
    }
};

Context &ctx() {
    static Context c;
    return c;
}

// The engine's buffers, stream and events belong to the device that was
// current at its first call.  Every entry point that touches them makes that
// device current for the call and gives the caller's back afterwards, so a
// thread that has switched to another device neither fails nor leaks work
// onto the wrong one.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard &) = delete;
    DeviceGuard &operator=(const DeviceGuard &) = delete;
};

int arith_code(Precision p) { return p == Precision::C128 ? 0 : (p == Precision::C128DF ? 1 : 2); }

// The planner configuration of a plan whose problems are added: the
// process-wide knobs (pqg_set_tuning), and for every knob left at its default
// there, the first autotuned entry matching the plan's form, arithmetic,
// largest column count, total steps and problem count.  Caller holds C.mu or
// C.cfg_mu.
PlanConfig tuned_config(const Context &C, const Planner &pl, Precision prec) {
    PlanConfig cfg = C.cfg;
    if (pl.form() == Form::LAPLACE) cfg.p_max = std::min<int64_t>(cfg.p_max, 512);  // Laplace tables
    if (C.tune.empty()) return cfg;
    int ncmax = 0;
    double steps = 0.0;
    int64_t probs = 0;
    for (const PendingProblem &p : pl.pending)
        if (p.kind == PQG_KIND_WALK) {
            ncmax = std::max(ncmax, p.nc);
            steps += p.S;
            ++probs;
        }
    if (probs == 0) return cfg;
    const int form = pl.form() == Form::LAPLACE ? 1 : 0, arith = arith_code(prec);
    for (const TuneEntry &t : C.tune) {
        if (t.form != form || t.arith != arith || ncmax < t.nc_lo || ncmax > t.nc_hi || steps < t.steps_lo ||
            steps >= t.steps_hi || probs < t.probs_lo || probs > t.probs_hi)
            continue;
        if (cfg.items_per_smsp == 0 && t.items_per_smsp > 0) cfg.items_per_smsp = t.items_per_smsp;
        if (!cfg.p_max_user && t.p_max > 0) {
            cfg.p_max = form == 1 ? std::min<int64_t>(t.p_max, 512) : t.p_max;
            cfg.p_max_user = true;
        }
        if (cfg.seed_steps == 0 && t.seed_steps > 0) cfg.seed_steps = t.seed_steps;
        if (t.blocks_per_sm > 0) cfg.blocks_per_sm = t.blocks_per_sm;
        break;
    }
    return cfg;
}

// The tuned configurations of a plan whose problems are added: its
// arithmetic's and the FP64 fallback's.  Initialises the context on first
// use; otherwise reads only the configuration, under cfg_mu.
int planning_configs(Context &C, const Planner &pl, Precision prec, PlanConfig &cfg, PlanConfig &cfg64) {
    if (!C.ready.load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> lock(C.mu);
        const int st = C.init();
        if (st) return st;
    }
    std::lock_guard<std::mutex> lock(C.cfg_mu);
    cfg = tuned_config(C, pl, prec);
    cfg64 = tuned_config(C, pl, Precision::C128);
    return PQG_OK;
}

// walk kernel for (form, precision, exact column count); `which` indexes the
// occupancy cache
const KernelInfo &kernel_for_plan(Form form, Precision prec, int nc, bool all_ones, bool pairs, int *which) {
    if (form == Form::PLAIN) {
        if (prec == Precision::C128DF) {
            *which = all_ones ? 8 : 4;
            return all_ones ? kernel_for(k_plain_dfo_0, k_plain_dfo_1, nc) : kernel_for(k_plain_df_0, k_plain_df_1, nc);
        }
        if (prec == Precision::C128) {
            *which = all_ones ? 6 : 0;
            return all_ones ? kernel_for(k_plain_c128o_0, k_plain_c128o_1, nc)
                            : kernel_for(k_plain_c128_0, k_plain_c128_1, nc);
        }
        *which = all_ones ? 7 : 1;
        return all_ones ? kernel_for(k_plain_c64o_0, k_plain_c64o_1, nc) : kernel_for(k_plain_c64_0, k_plain_c64_1, nc);
    }
    if (prec == Precision::C64) {
        if (pairs) {  // unit columns, two codes per iteration from a code-pair table
            *which = 5;
            return kernel_for(k_laplace_c64o_0, k_laplace_c64o_1, nc);
        }
        *which = 3;
        return kernel_for(k_laplace_c64_0, k_laplace_c64_1, nc);
    }
    if (prec == Precision::C128DF) {
        // the all-ones instantiations spill above 25 columns; the general ones
        // (multiplicities read from the problem record) do not
        const bool ones = all_ones && nc <= 25;
        *which = ones ? 9 : 10;
        return ones ? kernel_for(k_laplace_dfo_0, k_laplace_dfo_1, nc) : kernel_for(k_laplace_df_0, k_laplace_df_1, nc);
    }
    *which = 2;
    return kernel_for(k_laplace_c128_0, k_laplace_c128_1, nc);
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte layout of a packed plan (problems | item_begin | chunks | arena, the
// uploaded `total` bytes, then the device-built per-problem data up to
// `dev_total`) and of its outputs (values in the output type, then the low
// words in FP64).
struct PlanLayout {
    int64_t n_probs = 0;
    size_t o_probs = 0, o_items = 0, o_chunks = 0, o_arena = 0, total = 0, dev_total = 0;
    size_t out_bytes = 0, lo_bytes = 0;
};

// prefix-table entry: double2 (FP64), float4 (double-float), float2 (complex64
// Laplace) or float4 {re, re, im, im} (complex64 plain: the packed two-seed walk)
size_t delta_elem_bytes(const Planner &pl) {
    return (pl.precision() == Precision::C64 && pl.form() == Form::LAPLACE) ? 8 : 16;
}

PlanLayout layout_of(const Planner &pl, size_t out_elem) {
    PlanLayout L;
    L.n_probs = static_cast<int64_t>(pl.probs.size());
    L.o_probs = 0;
    L.o_items = align256(L.o_probs + sizeof(PqgProblem) * L.n_probs);
    L.o_chunks = align256(L.o_items + sizeof(int64_t) * (L.n_probs + 1));
    L.o_arena = align256(L.o_chunks + sizeof(PqgChunk) * std::max<size_t>(1, pl.chunks.size()));
    L.total = align256(L.o_arena + pl.arena.size());  // the arena ends 256-aligned: pdata starts here
    L.dev_total = L.total + align256(static_cast<size_t>(pl.pdata_bytes));
    L.out_bytes = static_cast<size_t>(pl.total_outputs) * 2 * out_elem;
    L.lo_bytes = static_cast<size_t>(pl.total_outputs) * 2 * sizeof(double);
    return L;
}

void pack_plan(const Planner &pl, const PlanLayout &L, unsigned char *h) {
    std::memcpy(h + L.o_probs, pl.probs.data(), sizeof(PqgProblem) * L.n_probs);
    std::memcpy(h + L.o_items, pl.item_begin.data(), sizeof(int64_t) * (L.n_probs + 1));
    if (!pl.chunks.empty()) std::memcpy(h + L.o_chunks, pl.chunks.data(), sizeof(PqgChunk) * pl.chunks.size());
    if (!pl.arena.empty()) std::memcpy(h + L.o_arena, pl.arena.data(), pl.arena.size());
}

int ensure_buffers(DeviceBuffers &B, const Planner &pl, const PlanLayout &L) {
    PQG_CUDA(B.plan.ensure(L.dev_total));
    const size_t n_parts = static_cast<size_t>(std::max<int64_t>(1, pl.total_parts));
    PQG_CUDA(B.partials.ensure(n_parts * 4 * sizeof(double)));
    PQG_CUDA(B.chunk_out.ensure(std::max<size_t>(1, pl.chunks.size()) * PQG_MAX_OUT * 4 * sizeof(double)));
    PQG_CUDA(B.out.ensure(align256(L.out_bytes) + L.lo_bytes));
    PQG_CUDA(B.counter.ensure(256));
    PQG_CUDA(B.delta.ensure(std::max<size_t>(1, static_cast<size_t>(pl.total_delta)) * delta_elem_bytes(pl)));
    return PQG_OK;
}

// Builds every problem's seeds, step rows and prefix tables of an uploaded
// plan (one launch; none without a walk).
int enqueue_prep(Context &C, DeviceBuffers &B, const Planner &pl, const PlanLayout &L, cudaStream_t s) {
    if (pl.total_items <= 0) return PQG_OK;
    unsigned char *d = static_cast<unsigned char *>(B.plan.p);
    PrepArgs A;
    A.probs = reinterpret_cast<PqgProblem *>(d + L.o_probs);
    A.arena = d + L.o_arena;
    A.delta = B.delta.p;
    A.matrix_off = pl.matrix_off;
    A.mat_cols = pl.mat_cols;
    A.n_probs = static_cast<int32_t>(L.n_probs);
    A.dup = (pl.precision() == Precision::C64 && pl.form() == Form::PLAIN) ? 1 : 0;
    A.pairs = pl.pairs ? 1 : 0;
    // enough blocks for every SM: several slices per problem for small batches
    const int64_t want = int64_t(C.num_sms) * 4;
    A.slices = static_cast<int32_t>(std::max<int64_t>(1, std::min<int64_t>(64, want / std::max<int64_t>(1, L.n_probs))));
    const int64_t blocks = std::min<int64_t>(L.n_probs * A.slices, int64_t(C.num_sms) * 16);
    switch (pl.precision()) {
        case Precision::C128:
            prep_problems<PREP_F64><<<blocks, 256, 0, s>>>(A);
            break;
        case Precision::C64:
            prep_problems<PREP_F32><<<blocks, 256, 0, s>>>(A);
            break;
        default:
            prep_problems<PREP_DF><<<blocks, 256, 0, s>>>(A);
    }
    PQG_CUDA(cudaGetLastError());
    g_launches++;
    return PQG_OK;
}

// Walk kernel of a plan, its dynamic shared memory set up, and its grid size.
int walk_launch_config(Context &C, const Planner &pl, const KernelInfo **k, int64_t *blocks) {
    int which = 0;
    const KernelInfo &kk = kernel_for_plan(pl.form(), pl.precision(), pl.max_nc, pl.all_ones, pl.pairs, &which);
    int &occ = C.occ_cache[which][pl.max_nc];
    if (occ < 0) {
        if (kk.smem_bytes > 0)
            PQG_CUDA(cudaFuncSetAttribute(kk.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(kk.smem_bytes)));
        int b = 0;
        PQG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kk.fn, PQG_WALK_THREADS, kk.smem_bytes));
        occ = std::max(1, b);
    }
    const int64_t warps_per_block = PQG_WALK_THREADS / 32;
    const int bps = C.blocks_per_sm > 0 ? C.blocks_per_sm : pl.config().blocks_per_sm;
    int64_t nb = static_cast<int64_t>(C.num_sms) * std::min(occ, bps > 0 ? bps : occ);
    nb = std::min<int64_t>(nb, (pl.total_items + warps_per_block - 1) / warps_per_block);
    *k = &kk;
    *blocks = std::max<int64_t>(1, nb);
    return PQG_OK;
}

// Enqueues the device pipeline of an uploaded plan on stream s: zero the
// queue head, walk, level-1 and level-2 reductions.  ev_w0 / ev_w1 (nullable)
// bracket the walk kernel.  Captured as is into a CUDA graph by plan handles.
template <typename T>
int enqueue_pipeline(Context &C, DeviceBuffers &B, const Planner &pl, const PlanLayout &L, cudaStream_t s,
                     cudaEvent_t ev_w0, cudaEvent_t ev_w1, const KernelInfo *k, int64_t blocks) {
    unsigned char *d = static_cast<unsigned char *>(B.plan.p);
    WalkArgs A;
    A.probs = reinterpret_cast<const PqgProblem *>(d + L.o_probs);
    A.item_begin = reinterpret_cast<const int64_t *>(d + L.o_items);
    A.arena = d + L.o_arena;
    A.delta = B.delta.p;
    A.counter = static_cast<unsigned long long *>(B.counter.p);
    A.partials = static_cast<double *>(B.partials.p);
    A.total_items = pl.total_items;
    A.n_probs = static_cast<int32_t>(L.n_probs);
    A.pad = 0;
    if (pl.total_items > 0) {
        PQG_CUDA(cudaMemsetAsync(B.counter.p, 0, sizeof(unsigned long long), s));
        void *args[] = {&A};
        if (ev_w0) PQG_CUDA(cudaEventRecord(ev_w0, s));
        PQG_CUDA(cudaLaunchKernel(k->fn, dim3(static_cast<unsigned>(blocks)), dim3(PQG_WALK_THREADS), args,
                                  k->smem_bytes, s));
        if (ev_w1) PQG_CUDA(cudaEventRecord(ev_w1, s));
        if (!pl.chunks.empty()) {
            const int n_chunks = static_cast<int>(pl.chunks.size());
            reduce_chunks<<<static_cast<unsigned>((n_chunks + 3) / 4), 128, 0, s>>>(
                reinterpret_cast<const PqgChunk *>(d + L.o_chunks), n_chunks, A.probs, A.partials,
                static_cast<double *>(B.chunk_out.p));
            PQG_CUDA(cudaGetLastError());
        }
    }
    unsigned char *dout = static_cast<unsigned char *>(B.out.p);
    double *dlo = reinterpret_cast<double *>(dout + align256(L.out_bytes));
    finish_problems<T><<<static_cast<unsigned>((L.n_probs + 3) / 4), 128, 0, s>>>(
        A.probs, static_cast<int>(L.n_probs), static_cast<const double *>(B.chunk_out.p), reinterpret_cast<T *>(dout),
        dlo);
    PQG_CUDA(cudaGetLastError());
    return PQG_OK;
}

// kernels one pipeline launches
int64_t pipeline_launches(const Planner &pl) {
    return 1 + (pl.total_items > 0 ? 1 : 0) + (pl.total_items > 0 && !pl.chunks.empty() ? 1 : 0);
}

// A sampler step fused behind a Laplace plan: one uniform in, one output mode
// out per problem (draw.cuh).
struct DrawRequest {
    const double *uniforms;
    int32_t *modes;
};

// Runs a finished plan; writes n_outputs complex values (2*T each) to host `out`
// and, if out_lo != nullptr, the low words (2 doubles per output).  With a
// draw request the outputs stay on the device and only the drawn modes come
// back.
template <typename T>
int run_plan(Context &C, Planner &pl, T *out, double *out_lo, const DrawRequest *draw = nullptr) {
    if (pl.probs.empty()) return PQG_OK;
    DeviceGuard dg(C.device);
    const PlanLayout L = layout_of(pl, sizeof(T));
    PQG_CUDA(C.h_plan.ensure(L.total));
    pack_plan(pl, L, static_cast<unsigned char *>(C.h_plan.p));
    int st = ensure_buffers(C.bufs, pl, L);
    if (st) return st;
    PQG_CUDA(C.h_out.ensure(align256(L.out_bytes) + L.lo_bytes));
    const KernelInfo *k = nullptr;
    int64_t blocks = 1;
    g_last_table = -1;
    g_last_nc = 0;
    if (pl.total_items > 0) {
        st = walk_launch_config(C, pl, &k, &blocks);
        if (st) return st;
        kernel_for_plan(pl.form(), pl.precision(), pl.max_nc, pl.all_ones, pl.pairs, &g_last_table);
        g_last_nc = pl.max_nc;
    }
    cudaStream_t s = C.stream;
    PQG_CUDA(cudaMemcpyAsync(C.bufs.plan.p, C.h_plan.p, L.total, cudaMemcpyHostToDevice, s));
    g_walk_ms = 0.0;
    g_dev_ms = 0.0;
    g_walk_steps = pl.total_steps;
    g_walk_flops = pl.total_flops;
    g_h2d = static_cast<double>(L.total);
    g_d2h = static_cast<double>(align256(L.out_bytes) + L.lo_bytes);
    PQG_CUDA(cudaEventRecord(C.evs, s));  // device time includes the prep kernel
    st = enqueue_prep(C, C.bufs, pl, L, s);
    if (st) return st;
    st = enqueue_pipeline<T>(C, C.bufs, pl, L, s, C.ev0, C.ev1, k, blocks);
    if (st) return st;
    g_launches += pipeline_launches(pl);
    if (draw) {
        const int64_t np = L.n_probs;
        const size_t ub = align256(sizeof(double) * np);
        PQG_CUDA(C.bufs.draw.ensure(ub + sizeof(int32_t) * np));
        PQG_CUDA(C.h_out.ensure(ub + sizeof(int32_t) * np));
        unsigned char *hd = static_cast<unsigned char *>(C.h_out.p);
        std::memcpy(hd, draw->uniforms, sizeof(double) * np);
        unsigned char *dd = static_cast<unsigned char *>(C.bufs.draw.p);
        PQG_CUDA(cudaMemcpyAsync(dd, hd, sizeof(double) * np, cudaMemcpyHostToDevice, s));
        unsigned char *dplan = static_cast<unsigned char *>(C.bufs.plan.p);
        draw_modes<T><<<static_cast<unsigned>((np + 3) / 4), 128, 0, s>>>(
            reinterpret_cast<const PqgProblem *>(dplan + L.o_probs), static_cast<int>(np), dplan + L.o_arena,
            pl.matrix_off, pl.mat_rows, pl.mat_cols, static_cast<const T *>(C.bufs.out.p),
            reinterpret_cast<const double *>(dd), reinterpret_cast<int32_t *>(dd + ub));
        PQG_CUDA(cudaGetLastError());
        g_launches++;
        PQG_CUDA(cudaEventRecord(C.ev2, s));
        PQG_CUDA(cudaMemcpyAsync(hd + ub, dd + ub, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, s));
        PQG_CUDA(cudaStreamSynchronize(s));
        if (pl.total_items > 0) {
            float ms = 0.0f;
            PQG_CUDA(cudaEventElapsedTime(&ms, C.ev0, C.ev1));
            g_walk_ms = ms;
        }
        float ms = 0.0f;
        PQG_CUDA(cudaEventElapsedTime(&ms, C.evs, C.ev2));
        g_dev_ms = ms;
        g_h2d += static_cast<double>(sizeof(double) * np);
        g_d2h = static_cast<double>(sizeof(int32_t) * np);
        std::memcpy(draw->modes, hd + ub, sizeof(int32_t) * np);
        return PQG_OK;
    }
    PQG_CUDA(cudaEventRecord(C.ev2, s));
    unsigned char *hout = static_cast<unsigned char *>(C.h_out.p);
    PQG_CUDA(cudaMemcpyAsync(hout, C.bufs.out.p, align256(L.out_bytes) + L.lo_bytes, cudaMemcpyDeviceToHost, s));
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
    std::memcpy(out, hout, L.out_bytes);
    if (out_lo) std::memcpy(out_lo, hout + align256(L.out_bytes), L.lo_bytes);
    return PQG_OK;
}

std::vector<double> widen(const float *m, int64_t n) {
    std::vector<double> v(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) v[i] = static_cast<double>(m[i]);
    return v;
}

// Precision of a complex128 call: the explicit mode, else PQG_C128_MODE from the
// environment ("fp64", "df" or "auto"), else auto (double-float where valid).
Precision c128_precision(int32_t mode) {
    if (mode == PQG_MODE_FP64) return Precision::C128;
    if (mode == PQG_MODE_DF) return Precision::C128DF;
    const char *env = std::getenv("PQG_C128_MODE");
    if (env && std::strcmp(env, "fp64") == 0) return Precision::C128;
    return Precision::C128DF;
}

// Whether a complex128 plain plan chosen by `auto` (double-float) runs the
// FP64 walk instead: outside the double-float domain, or so small (at most
// 2^16 Gray-code steps in all) that the FP64 walk costs microseconds -- it
// then keeps FP64's accuracy, where the double-float walk rounds each scaled
// matrix entry to 2^-47 once (relative 1e-14 on a 1 x 1 permanent).
bool use_fp64_walk(const Planner &pl, int32_t mode) {
    if (pl.precision() != Precision::C128DF) return false;
    if (!pl.df_ok) return true;
    if (mode == PQG_MODE_DF) return false;
    const char *env = std::getenv("PQG_C128_MODE");
    if (env && std::strcmp(env, "df") == 0) return false;
    return pl.total_steps <= 65536.0;
}

template <typename T>
int plain_batch(const double *matrix, int64_t nr, int64_t nc, const int32_t *rows, const int32_t *cols, int64_t batch,
                Precision prec, T *out, double *out_lo, int32_t mode = PQG_MODE_AUTO) {
    if (batch < 0 || nr < 0 || nc < 0 || !out) return fail(PQG_ERR_INVALID, "invalid arguments");
    Context &C = ctx();
    // Host planning runs outside the context lock (threads plan concurrently;
    // only the device part is serialised); inputs are validated before the
    // device is touched.
    Planner pl(prec, Form::PLAIN, PlanConfig{});
    pl.set_matrix(matrix, nr, nc);
    {
        std::string err;
        int64_t bad = 0;
        int st = pl.add_batch(rows, cols, batch, err, &bad);
        if (st) return fail(st, batch > 1 ? "problem " + std::to_string(bad) + ": " + err : err);
    }
    PlanConfig cfg, cfg64;
    {
        const int st = planning_configs(C, pl, prec, cfg, cfg64);
        if (st) return st;
    }
    pl.set_config(cfg);
    pl.finish();
    if (use_fp64_walk(pl, mode)) {
        // outside the double-float domain, or a small plan: the FP64 walk
        pl.set_precision(Precision::C128);
        pl.set_config(cfg64);
        pl.finish();
    }
    std::lock_guard<std::mutex> lock(C.mu);
    return run_plan<T>(C, pl, out, out_lo);
}

// The double-float Laplace walk serves plans in the double-float domain; any
// other complex128 Laplace plan is redone for the FP64 walk.
void laplace_precision_fallback(Planner &pl, const PlanConfig &cfg64) {
    if (pl.precision() == Precision::C128DF && !pl.df_ok) {
        pl.set_precision(Precision::C128);
        pl.set_config(cfg64);
        pl.finish();
    }
}

// Plans `batch` Laplace problems over one matrix (outside the context lock).
int plan_laplace(Context &C, Planner &pl, const double *matrix, int64_t nr, int64_t nc, const int32_t *rows,
                 const int32_t *cols, int64_t batch) {
    pl.set_matrix(matrix, nr, nc);
    {
        std::string err;
        int64_t bad = 0;
        int st = pl.add_batch(rows, cols, batch, err, &bad);
        if (st) return fail(st, batch > 1 ? "problem " + std::to_string(bad) + ": " + err : err);
    }
    PlanConfig cfg, cfg64;
    {
        const int st = planning_configs(C, pl, pl.precision(), cfg, cfg64);
        if (st) return st;
    }
    pl.set_config(cfg);
    pl.finish();
    laplace_precision_fallback(pl, cfg64);
    return PQG_OK;
}

// One step of the batched exact sampler: the Laplace permanents of shot b
// (rows = its output photons so far, cols = its input photons so far) and the
// draw of its next output mode with uniforms[b] (draw.cuh).
template <typename T>
int sampler_step(const double *matrix, int64_t nr, int64_t nc, const int32_t *rows, const int32_t *cols,
                 int64_t batch, Precision prec, const double *uniforms, int32_t *modes) {
    if (nr <= 0 || nc < 0 || batch < 0 || (batch > 0 && (!uniforms || !modes)))
        return fail(PQG_ERR_INVALID, "invalid arguments");
    if (nr > (int64_t(1) << 31) - 1) return fail(PQG_ERR_TOO_LARGE, "more than 2^31 - 1 output modes");
    if (batch == 0) return PQG_OK;
    Context &C = ctx();
    Planner pl(prec, Form::LAPLACE, PlanConfig{});
    int st = plan_laplace(C, pl, matrix, nr, nc, rows, cols, batch);
    if (st) return st;
    for (int64_t b = 0; b < batch; ++b)
        if (pl.pending[static_cast<size_t>(b)].kind != PQG_KIND_WALK)
            return fail(PQG_ERR_INVALID, "shot " + std::to_string(b) +
                                             ": a sampler step needs at least one output and one input photon");
    DrawRequest dr{uniforms, modes};
    std::lock_guard<std::mutex> lock(C.mu);
    return run_plan<T>(C, pl, nullptr, nullptr, &dr);
}

// Laplace permanents of `batch` problems sharing one matrix; problem b writes
// 2*nc values at out + 2*nc*b (its count, 1 or nc, to n_out[b]).
template <typename T>
int laplace_batch(const double *matrix, int64_t nr, int64_t nc, const int32_t *rows, const int32_t *cols,
                  int64_t batch, Precision prec, T *out, int64_t *n_out) {
    if (nr < 0 || nc < 0 || batch < 0 || !out) return fail(PQG_ERR_INVALID, "invalid arguments");
    Context &C = ctx();
    // planning and the scatter of the outputs run outside the context lock
    Planner pl(prec, Form::LAPLACE, PlanConfig{});
    int st = plan_laplace(C, pl, matrix, nr, nc, rows, cols, batch);
    if (st) return st;
    std::vector<T> res(2 * static_cast<size_t>(std::max<int64_t>(1, pl.total_outputs)));
    {
        std::lock_guard<std::mutex> lock(C.mu);
        int st = run_plan<T>(C, pl, res.data(), nullptr);
        if (st) return st;
    }
    const int64_t stride = 2 * std::max<int64_t>(1, nc);
    std::vector<int> slot(static_cast<size_t>(std::max<int64_t>(1, nc)));
    for (int64_t b = 0; b < batch; ++b) {
        const PendingProblem &pp = pl.pending[static_cast<size_t>(b)];
        const int64_t oi = pl.out_of[static_cast<size_t>(b)];
        T *o = out + b * stride;
        if (pp.kind == PQG_KIND_CONSTANT) {
            for (int64_t j = 0; j < stride; ++j) o[j] = T(0);
            o[0] = res[2 * oi];
            o[1] = res[2 * oi + 1];
            if (n_out) n_out[b] = 1;
            continue;
        }
        laplace_slots(pp, nc, slot.data());
        for (int64_t j = 0; j < nc; ++j) {
            o[2 * j] = res[2 * (oi + slot[j])];
            o[2 * j + 1] = res[2 * (oi + slot[j]) + 1];
        }
        if (n_out) n_out[b] = nc;
    }
    return PQG_OK;
}

// Gradient of the permanent with respect to every matrix entry, for `batch`
// matrices stacked as (batch, nr, nc), each with its own multiplicities:
//     G_ij = rows_i cols_j perm(A; rows - e_i, cols - e_j)
// (the reference's grad_perm, src/permanent.cpp:271-300, which evaluates the
// n^2 minors one by one).  Here one Laplace plan serves every matrix: problem
// (b, i) walks rows - e_i once and its output j is perm(A_b; rows - e_i,
// cols - e_j) (Lemma 1 of arXiv:2005.04214), so a matrix costs one walk per
// row with nonzero multiplicity.  Entries with rows_i = 0 or cols_j = 0 are 0;
// unequal sums fail as the reference's first minor would (only when some
// entry has rows_i > 0 and cols_j > 0).  out: batch x nr x nc complex.
template <typename T>
int grad_batch(const double *mats, int64_t nr, int64_t nc, const int32_t *rows, const int32_t *cols, int64_t batch,
               Precision prec, T *out) {
    if (nr < 0 || nc < 0 || batch < 0 || !out || (batch * nr * nc > 0 && !mats) || (batch * nr > 0 && !rows) ||
        (batch * nc > 0 && !cols))
        return fail(PQG_ERR_INVALID, "invalid arguments");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    const size_t per = static_cast<size_t>(nr * nc) * 2;
    std::fill(out, out + per * static_cast<size_t>(batch), T(0));
    PlanConfig cfg = C.cfg;
    cfg.p_max = std::min<int64_t>(cfg.p_max, 512);
    Planner pl(prec, Form::LAPLACE, cfg);
    pl.set_matrix(mats, batch * nr, nc);
    struct Minor {
        int64_t b, i;
    };
    std::vector<Minor> minors;
    std::vector<int32_t> r2(static_cast<size_t>(nr));
    for (int64_t b = 0; b < batch; ++b) {
        const int32_t *rb = rows + b * nr, *cb = cols + b * nc;
        int64_t sr = 0, sc = 0, i_any = -1, j_any = -1;
        for (int64_t i = 0; i < nr; ++i) {
            if (rb[i] < 0) return fail(PQG_ERR_INVALID, "row multiplicities must be nonnegative");
            sr += rb[i];
            if (rb[i] > 0) i_any = i;
        }
        for (int64_t j = 0; j < nc; ++j) {
            if (cb[j] < 0) return fail(PQG_ERR_INVALID, "column multiplicities must be nonnegative");
            sc += cb[j];
            if (cb[j] > 0) j_any = j;
        }
        if (i_any < 0 || j_any < 0) continue;  // every entry is 0
        if (sr != sc) {
            std::string msg = "Number of input and output states should be equal";
            return fail(PQG_ERR_SUM_MISMATCH, batch > 1 ? "matrix " + std::to_string(b) + ": " + msg : msg);
        }
        if (sr == 1) {  // the single minor is the empty matrix: perm = 1
            out[static_cast<size_t>(b) * per + 2 * (i_any * nc + j_any)] = T(1);
            continue;
        }
        for (int64_t i = 0; i < nr; ++i) {
            if (rb[i] == 0) continue;
            std::copy(rb, rb + nr, r2.begin());
            r2[i] -= 1;
            std::string err;
            int st = pl.add(r2.data(), cb, err, b * nr, nr);
            if (st) return fail(st, batch > 1 ? "matrix " + std::to_string(b) + ": " + err : err);
            minors.push_back({b, i});
        }
    }
    if (minors.empty()) return PQG_OK;
    int st = C.init();
    if (st) return st;
    pl.set_config(tuned_config(C, pl, pl.precision()));
    pl.finish();
    laplace_precision_fallback(pl, tuned_config(C, pl, Precision::C128));
    std::vector<T> res(2 * static_cast<size_t>(std::max<int64_t>(1, pl.total_outputs)));
    st = run_plan<T>(C, pl, res.data(), nullptr);
    if (st) return st;
    std::vector<int> slot(static_cast<size_t>(std::max<int64_t>(1, nc)));
    for (size_t q = 0; q < minors.size(); ++q) {
        const Minor &mi = minors[q];
        const PendingProblem &pp = pl.pending[q];
        laplace_slots(pp, nc, slot.data());
        const int64_t oi = pl.out_of[q];
        const int32_t *rb = rows + mi.b * nr, *cb = cols + mi.b * nc;
        T *o = out + static_cast<size_t>(mi.b) * per + 2 * mi.i * nc;
        for (int64_t j = 0; j < nc; ++j) {
            if (cb[j] == 0) continue;
            const double f = static_cast<double>(rb[mi.i]) * static_cast<double>(cb[j]);
            o[2 * j] = static_cast<T>(f * static_cast<double>(res[2 * (oi + slot[j])]));
            o[2 * j + 1] = static_cast<T>(f * static_cast<double>(res[2 * (oi + slot[j]) + 1]));
        }
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
    PQG_CUDA(C.bufs.out.ensure(1024));
    F *o = static_cast<F *>(C.bufs.out.p);
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

// ------------------------------------------------------------ plan handles
// A plan handle owns a planned, uploaded batch, its device buffers, a stream
// and a CUDA graph of its device pipeline, so that repeated executions cost
// one graph launch (no planning, no copies).
struct PlanHandle {
    PlanHandle(Precision prec, Form form, const PlanConfig &cfg) : pl(prec, form, cfg) {}
    Planner pl;
    PlanLayout L;
    DeviceBuffers B;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool single = false;      // complex64 outputs
    bool launched = false;
    int device = 0;           // the engine's device, where the handle's buffers live
    bool on_device = false;   // plan_build ran: device resources to free
    int64_t n_cols = 0;       // Laplace: outputs per problem in the caller's layout
    ~PlanHandle() {
        if (!on_device) return;
        DeviceGuard dg(device);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
        for (DevBuf *b : {&B.plan, &B.partials, &B.chunk_out, &B.out, &B.counter, &B.delta})
            if (b->p) cudaFree(b->p);
    }
};

template <typename T>
int plan_build(Context &C, PlanHandle *h) {
    h->device = C.device;
    h->on_device = true;
    DeviceGuard dg(C.device);
    h->L = layout_of(h->pl, sizeof(T));
    int st = ensure_buffers(h->B, h->pl, h->L);
    if (st) return st;
    PQG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    PQG_CUDA(cudaEventCreate(&h->e0));
    PQG_CUDA(cudaEventCreate(&h->e1));
    std::vector<unsigned char> hp(h->L.total);
    pack_plan(h->pl, h->L, hp.data());
    PQG_CUDA(cudaMemcpyAsync(h->B.plan.p, hp.data(), h->L.total, cudaMemcpyHostToDevice, h->stream));
    st = enqueue_prep(C, h->B, h->pl, h->L, h->stream);
    if (st) return st;
    PQG_CUDA(cudaStreamSynchronize(h->stream));
    const KernelInfo *k = nullptr;
    int64_t blocks = 1;
    if (h->pl.total_items > 0) {
        st = walk_launch_config(C, h->pl, &k, &blocks);
        if (st) return st;
    }
    PQG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    st = enqueue_pipeline<T>(C, h->B, h->pl, h->L, h->stream, nullptr, nullptr, k, blocks);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return fail(PQG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    h->graph = g;
    PQG_CUDA(cudaGraphInstantiate(&h->exec, h->graph, 0));
    return PQG_OK;
}

}  // namespace

void set_last_error(const char *msg) { g_err = msg; }

}  // namespace pqg

using namespace pqg;

extern "C" {

const char *pqg_last_error(void) { return g_err.c_str(); }

const char *pqg_version(void) { return "pqperm_gb300 0.1.0 (sm_103a)"; }

uint64_t pqg_kernel_launches(void) { return g_launches.load(); }

int pqg_permanent_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows, const int32_t *cols,
                       int32_t mode, double *out, double *out_lo) try {
    return plain_batch<double>(matrix, n_rows, n_cols, rows, cols, 1, c128_precision(mode), out, out_lo, mode);
} catch (...) {
    return host_failure();
}

int pqg_permanent_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows, const int32_t *cols,
                      float *out) try {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return plain_batch<float>(m.data(), n_rows, n_cols, rows, cols, 1, Precision::C64, out, nullptr);
} catch (...) {
    return host_failure();
}

int pqg_permanent_batch_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                             const int32_t *cols, int64_t batch, int32_t mode, double *out) try {
    return plain_batch<double>(matrix, n_rows, n_cols, rows, cols, batch, c128_precision(mode), out, nullptr, mode);
} catch (...) {
    return host_failure();
}

int pqg_permanent_batch_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                            const int32_t *cols, int64_t batch, float *out) try {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return plain_batch<float>(m.data(), n_rows, n_cols, rows, cols, batch, Precision::C64, out, nullptr);
} catch (...) {
    return host_failure();
}

int pqg_permanent_laplace_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                               const int32_t *cols, double *out, int64_t *n_out) try {
    return laplace_one<double>(matrix, n_rows, n_cols, rows, cols, c128_precision(PQG_MODE_AUTO), out, n_out);
} catch (...) {
    return host_failure();
}

int pqg_permanent_laplace_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                              const int32_t *cols, float *out, int64_t *n_out) try {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return laplace_one<float>(m.data(), n_rows, n_cols, rows, cols, Precision::C64, out, n_out);
} catch (...) {
    return host_failure();
}

int pqg_permanent_laplace_batch_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                                     const int32_t *cols, int64_t batch, double *out, int64_t *n_out) try {
    return laplace_batch<double>(matrix, n_rows, n_cols, rows, cols, batch, c128_precision(PQG_MODE_AUTO), out,
                                 n_out);
} catch (...) {
    return host_failure();
}

int pqg_permanent_laplace_batch_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                                    const int32_t *cols, int64_t batch, float *out, int64_t *n_out) try {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return laplace_batch<float>(m.data(), n_rows, n_cols, rows, cols, batch, Precision::C64, out, n_out);
} catch (...) {
    return host_failure();
}

int pqg_sampler_step_c128(const double *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                          const int32_t *cols, int64_t batch, const double *uniforms, int32_t *modes) try {
    return sampler_step<double>(matrix, n_rows, n_cols, rows, cols, batch, c128_precision(PQG_MODE_AUTO), uniforms,
                                modes);
} catch (...) {
    return host_failure();
}

int pqg_sampler_step_c64(const float *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                         const int32_t *cols, int64_t batch, const double *uniforms, int32_t *modes) try {
    if (n_rows < 0 || n_cols < 0) return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrix, 2 * n_rows * n_cols);
    return sampler_step<float>(m.data(), n_rows, n_cols, rows, cols, batch, Precision::C64, uniforms, modes);
} catch (...) {
    return host_failure();
}

int pqg_permanent_grad_c128(const double *matrices, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                            const int32_t *cols, int64_t batch, double *out) try {
    return grad_batch<double>(matrices, n_rows, n_cols, rows, cols, batch, c128_precision(PQG_MODE_AUTO), out);
} catch (...) {
    return host_failure();
}

int pqg_permanent_grad_c64(const float *matrices, int64_t n_rows, int64_t n_cols, const int32_t *rows,
                           const int32_t *cols, int64_t batch, float *out) try {
    if (n_rows < 0 || n_cols < 0 || batch < 0 || (batch * n_rows * n_cols > 0 && !matrices))
        return fail(PQG_ERR_INVALID, "invalid arguments");
    std::vector<double> m = widen(matrices, 2 * batch * n_rows * n_cols);
    return grad_batch<float>(m.data(), n_rows, n_cols, rows, cols, batch, Precision::C64, out);
} catch (...) {
    return host_failure();
}

int pqg_set_tuning(int64_t items_per_smsp, int64_t p_max, int64_t seed_steps) try {
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    std::lock_guard<std::mutex> cfg_lock(C.cfg_mu);
    if (items_per_smsp < 0 || p_max < 0 || p_max > 32768 || seed_steps < 0)
        return fail(PQG_ERR_INVALID, "invalid tuning values");
    PlanConfig d;
    C.cfg.items_per_smsp = items_per_smsp;  // 0: the per-arithmetic default
    C.cfg.p_max = p_max ? p_max : d.p_max;
    C.cfg.p_max_user = p_max != 0;
    C.cfg.seed_steps = seed_steps;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_get_tuning(int64_t *items_per_smsp, int64_t *p_max, int64_t *seed_steps) try {
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    if (items_per_smsp) *items_per_smsp = C.cfg.items_per_smsp;
    if (p_max) *p_max = C.cfg.p_max;
    if (seed_steps) *seed_steps = C.cfg.seed_steps;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_set_blocks_per_sm(int32_t blocks) try {
    if (blocks < 0 || blocks > 32) return fail(PQG_ERR_INVALID, "blocks per SM must be between 0 and 32");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    C.blocks_per_sm = blocks;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_tuning_add(int32_t form, int32_t arith, int32_t nc_lo, int32_t nc_hi, double steps_lo, double steps_hi,
                   int64_t probs_lo, int64_t probs_hi, int64_t items_per_smsp, int64_t p_max, int64_t seed_steps,
                   int32_t blocks_per_sm) try {
    if (form < 0 || form > 1 || arith < 0 || arith > 2 || nc_lo > nc_hi || !(steps_lo < steps_hi) ||
        probs_lo > probs_hi || items_per_smsp < 0 || p_max < 0 || p_max > 32768 || seed_steps < 0 ||
        blocks_per_sm < 0 || blocks_per_sm > 32)
        return fail(PQG_ERR_INVALID, "invalid tuning entry");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    std::lock_guard<std::mutex> cfg_lock(C.cfg_mu);
    C.tune.push_back(TuneEntry{form, arith, nc_lo, nc_hi, steps_lo, steps_hi, probs_lo, probs_hi, items_per_smsp,
                               p_max, seed_steps, blocks_per_sm});
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_tuning_clear(void) try {
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    std::lock_guard<std::mutex> cfg_lock(C.cfg_mu);
    C.tune.clear();
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_tuning_count(int64_t *count) try {
    if (!count) return fail(PQG_ERR_INVALID, "null output");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    *count = static_cast<int64_t>(C.tune.size());
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_plan_config(pqg_plan_t *plan, int64_t *items_per_smsp, int64_t *p_max, int64_t *seed_steps,
                    int32_t *blocks_per_sm) try {
    PlanHandle *h = reinterpret_cast<PlanHandle *>(plan);
    if (!h) return fail(PQG_ERR_INVALID, "null plan");
    const PlanConfig &c = h->pl.config();
    if (items_per_smsp) *items_per_smsp = c.items_per_smsp;
    if (p_max) *p_max = c.p_max;
    if (seed_steps) *seed_steps = c.seed_steps;
    if (blocks_per_sm) *blocks_per_sm = c.blocks_per_sm;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_device_info(char *name, int64_t name_len, int32_t *num_sms) try {
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    int st = C.init();
    if (st) return st;
    cudaDeviceProp prop;
    PQG_CUDA(cudaGetDeviceProperties(&prop, C.device));
    if (name && name_len > 0) {
        std::strncpy(name, prop.name, static_cast<size_t>(name_len - 1));
        name[name_len - 1] = '\0';
    }
    if (num_sms) *num_sms = C.num_sms;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_measure_vector_peaks(double ms, double *out2) try {
    if (!out2) return fail(PQG_ERR_INVALID, "null output");
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    int st = C.init();
    if (st) return st;
    DeviceGuard dg(C.device);
    st = time_fma<double, 8>(C, ms, &out2[0]);
    if (st) return st;
    return time_fma<float, 16>(C, ms, &out2[1]);
} catch (...) {
    return host_failure();
}

int pqg_last_timing(double *walk_ms, double *device_ms, double *steps, double *flops, double *h2d_bytes,
                    double *d2h_bytes) try {
    if (h2d_bytes) *h2d_bytes = g_h2d;
    if (d2h_bytes) *d2h_bytes = g_d2h;
    if (walk_ms) *walk_ms = g_walk_ms;
    if (device_ms) *device_ms = g_dev_ms;
    if (steps) *steps = g_walk_steps;
    if (flops) *flops = g_walk_flops;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_last_walk_kernel(int32_t *table, int32_t *n_cols) try {
    if (table) *table = g_last_table;
    if (n_cols) *n_cols = g_last_nc;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_plan_create(const void *matrix, int64_t n_rows, int64_t n_cols, const int32_t *rows, const int32_t *cols,
                    int64_t batch, int32_t dtype, int32_t form, int32_t mode, pqg_plan_t **out_plan) try {
    if (!out_plan || batch < 0 || n_rows < 0 || n_cols < 0 || (dtype != 0 && dtype != 1) || (form != 0 && form != 1))
        return fail(PQG_ERR_INVALID, "invalid arguments");
    *out_plan = nullptr;
    std::vector<double> widened;
    const double *m = static_cast<const double *>(matrix);
    if (dtype == 1) {
        widened = widen(static_cast<const float *>(matrix), 2 * n_rows * n_cols);
        m = widened.data();
    }
    Context &C = ctx();
    std::lock_guard<std::mutex> lock(C.mu);
    const Form fm = form == 1 ? Form::LAPLACE : Form::PLAIN;
    const Precision prec = dtype == 1 ? Precision::C64 : c128_precision(mode);
    PlanHandle *h = new PlanHandle(prec, fm, C.cfg);
    h->single = dtype == 1;
    h->n_cols = n_cols;
    h->pl.set_matrix(m, n_rows, n_cols);
    {
        std::string err;
        int64_t bad = 0;
        int st = h->pl.add_batch(rows, cols, batch, err, &bad);
        if (st) {
            delete h;
            return fail(st, batch > 1 ? "problem " + std::to_string(bad) + ": " + err : err);
        }
    }
    int st = C.init();
    if (st) {
        delete h;
        return st;
    }
    h->pl.set_config(tuned_config(C, h->pl, prec));
    h->pl.finish();
    if (fm == Form::LAPLACE) {
        laplace_precision_fallback(h->pl, tuned_config(C, h->pl, Precision::C128));
    } else if (use_fp64_walk(h->pl, mode)) {
        h->pl.set_precision(Precision::C128);
        h->pl.set_config(tuned_config(C, h->pl, Precision::C128));
        h->pl.finish();
    }
    st = h->single ? plan_build<float>(C, h) : plan_build<double>(C, h);
    if (st) {
        delete h;
        return st;
    }
    *out_plan = reinterpret_cast<pqg_plan_t *>(h);
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_plan_launch(pqg_plan_t *plan) try {
    PlanHandle *h = reinterpret_cast<PlanHandle *>(plan);
    if (!h) return fail(PQG_ERR_INVALID, "null plan");
    DeviceGuard dg(h->device);
    PQG_CUDA(cudaEventRecord(h->e0, h->stream));
    PQG_CUDA(cudaGraphLaunch(h->exec, h->stream));
    PQG_CUDA(cudaEventRecord(h->e1, h->stream));
    g_launches += pipeline_launches(h->pl);
    h->launched = true;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_plan_synchronize(pqg_plan_t *plan, double *device_ms) try {
    PlanHandle *h = reinterpret_cast<PlanHandle *>(plan);
    if (!h) return fail(PQG_ERR_INVALID, "null plan");
    DeviceGuard dg(h->device);
    PQG_CUDA(cudaStreamSynchronize(h->stream));
    if (device_ms) {
        float ms = 0.0f;
        if (h->launched) PQG_CUDA(cudaEventElapsedTime(&ms, h->e0, h->e1));
        *device_ms = ms;
    }
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_plan_read(pqg_plan_t *plan, void *out, int64_t *n_values) try {
    PlanHandle *h = reinterpret_cast<PlanHandle *>(plan);
    if (!h || !out) return fail(PQG_ERR_INVALID, "null argument");
    DeviceGuard dg(h->device);
    std::vector<unsigned char> tmp(h->L.out_bytes);
    if (h->L.out_bytes) {
        PQG_CUDA(cudaMemcpyAsync(tmp.data(), h->B.out.p, h->L.out_bytes, cudaMemcpyDeviceToHost, h->stream));
        PQG_CUDA(cudaStreamSynchronize(h->stream));
    }
    const size_t es = h->single ? sizeof(float) : sizeof(double);
    if (h->pl.form() == Form::PLAIN) {
        std::memcpy(out, tmp.data(), h->L.out_bytes);
        if (n_values) *n_values = static_cast<int64_t>(h->pl.probs.size());
        return PQG_OK;
    }
    // Laplace: scatter every problem's outputs to the caller's column layout
    const int64_t stride = std::max<int64_t>(1, h->n_cols);
    std::vector<int> slot(static_cast<size_t>(stride));
    unsigned char *o = static_cast<unsigned char *>(out);
    for (size_t b = 0; b < h->pl.pending.size(); ++b) {
        const PendingProblem &pp = h->pl.pending[b];
        const int64_t oi = h->pl.out_of[b];
        unsigned char *ob = o + b * stride * 2 * es;
        std::memset(ob, 0, stride * 2 * es);
        if (pp.kind == PQG_KIND_CONSTANT) {
            std::memcpy(ob, tmp.data() + oi * 2 * es, 2 * es);
            continue;
        }
        laplace_slots(pp, h->n_cols, slot.data());
        for (int64_t j = 0; j < h->n_cols; ++j)
            std::memcpy(ob + j * 2 * es, tmp.data() + (oi + slot[j]) * 2 * es, 2 * es);
    }
    if (n_values) *n_values = static_cast<int64_t>(h->pl.pending.size()) * stride;
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_plan_info(pqg_plan_t *plan, double *steps, double *flops, int64_t *work_items, int64_t *h2d_bytes) try {
    PlanHandle *h = reinterpret_cast<PlanHandle *>(plan);
    if (!h) return fail(PQG_ERR_INVALID, "null plan");
    if (steps) *steps = h->pl.total_steps;
    if (flops) *flops = h->pl.total_flops;
    if (work_items) *work_items = h->pl.total_items;
    if (h2d_bytes) *h2d_bytes = static_cast<int64_t>(h->L.total);
    return PQG_OK;
} catch (...) {
    return host_failure();
}

int pqg_plan_destroy(pqg_plan_t *plan) try {
    PlanHandle *h = reinterpret_cast<PlanHandle *>(plan);
    if (h) {
        cudaStreamSynchronize(h->stream);
        delete h;
    }
    return PQG_OK;
} catch (...) {
    return host_failure();
}

}  // extern "C"
