// Allocation-free permanent of a square matrix with every row and column taken
// once, for callers that cannot allocate device memory: code whose allocator
// has already claimed the GPU (frameworks that reserve most of the device up
// front), code on latency-critical paths where a device allocation's implicit
// synchronisation is not acceptable, or code running while the caller's own
// stream is being recorded.  The caller passes device pointers to its input and
// output and a stream; everything else the computation needs lives in one
// file-scope device array, the scratch below.
//
// The kernels are a variant of the FP64 walk (walk_plain.cuh): the Gray-code
// digits are all binary, so the plan is implicit and passed by value, the
// prefix table Delta(t) and the per-item partial sums go to the scratch, and a
// single block folds the partials in double-double.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/pqperm_gb300.h"
#include "walk_common.cuh"

namespace pqg {

void set_last_error(const char *msg);  // capi.cu: the message pqg_last_error() returns

namespace {

constexpr int kNoallocMaxN = PQG_NOALLOC_MAX_N;
constexpr size_t kScratchBytes = PQG_NOALLOC_SCRATCH_BYTES;

// The scratch of every call on this device.  In host code this name is only a
// stand-in for the device array; its device address comes from
// cudaGetSymbolAddress (scratch_address below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Implicit plan of an all-ones n x n permanent, passed by value.
struct UnitPlan {
    int n;          // matrix order
    int K;          // inner (binary) digits: P = 2^K inner codes
    int n_outer;    // outer digits: Q = 2^n_outer outer positions
    int R;          // outer positions per lane
    int64_t items;  // work items (32 lanes x R positions)
    int64_t off_delta, off_partials;  // byte offsets into the scratch
};

// Digit layout after the reference's reduction (src/permanent.cpp:54-95):
// row 0 is the prepended copy of matrix row 0 (multiplicity 1); matrix row 0
// keeps multiplicity 0 and drops out; matrix rows 1..n-1 are the binary
// digits: inner digits k = 0..K-1 are rows 1+k, outer digits o are rows 1+K+o.
__global__ void unit_build_delta(const double2 *__restrict__ a, UnitPlan p, unsigned char *__restrict__ scratch) {
    double2 *delta = reinterpret_cast<double2 *>(scratch + p.off_delta);
    const int64_t total = (int64_t(1) << p.K) * p.n;
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t t = e / p.n;
        const int j = static_cast<int>(e - t * p.n);
        const uint64_t g = static_cast<uint64_t>(t) ^ (static_cast<uint64_t>(t) >> 1);
        double re = 0.0, im = 0.0;
        for (int k = 0; k < p.K; ++k)
            if ((g >> k) & 1) {
                const double2 v = a[static_cast<int64_t>(1 + k) * p.n + j];
                re = __fma_rn(-2.0, v.x, re);
                im = __fma_rn(-2.0, v.y, im);
            }
        delta[e] = make_double2(re, im);
    }
}

__global__ void __launch_bounds__(PQG_WALK_THREADS, 2)
    unit_walk(const double2 *__restrict__ a, UnitPlan p, unsigned char *__restrict__ scratch) {
    unsigned long long *counter = reinterpret_cast<unsigned long long *>(scratch);
    const double2 *delta = reinterpret_cast<const double2 *>(scratch + p.off_delta);
    double *partials = reinterpret_cast<double *>(scratch + p.off_partials);
    const int n = p.n;
    const int P = 1 << p.K;
    const int64_t Q = int64_t(1) << p.n_outer;
    const int lane = threadIdx.x & 31;
    for (;;) {
        const int64_t item = next_item(counter, lane);
        if (item >= p.items) return;
        const int64_t r0 = (item * PQG_ITEM_LANES + lane) * p.R;
        ddv sr{0.0, 0.0}, si{0.0, 0.0};
        if (r0 < Q) {
            // FP64 seed at outer position r0: column sums minus twice the
            // rows of the outer digits set in its Gray code
            double cr[kNoallocMaxN], ci[kNoallocMaxN];
            const uint64_t g0 = static_cast<uint64_t>(r0) ^ (static_cast<uint64_t>(r0) >> 1);
#pragma unroll
            for (int j = 0; j < kNoallocMaxN; ++j) {
                if (j >= n) break;
                double re = 0.0, im = 0.0;
                for (int i = 0; i < n; ++i) {
                    const double2 v = a[static_cast<int64_t>(i) * n + j];
                    const bool outer_set = i >= 1 + p.K && ((g0 >> (i - 1 - p.K)) & 1);
                    const double f = outer_set ? -1.0 : 1.0;
                    re = __fma_rn(f, v.x, re);
                    im = __fma_rn(f, v.y, im);
                }
                cr[j] = re;
                ci[j] = im;
            }
            double wout = (__popcll(g0) & 1) ? -1.0 : 1.0;
            const int64_t my_R = (Q - r0 < p.R) ? (Q - r0) : p.R;
            for (int64_t seg = 0; seg < my_R; ++seg) {
                double ar = 0.0, ai = 0.0;
                for (int s = 0; s < P; ++s) {
                    const int t = (seg & 1) ? P - 1 - s : s;
                    const double2 *d = delta + static_cast<int64_t>(t) * n;
                    double xr = 1.0, xi = 0.0;
#pragma unroll
                    for (int j = 0; j < kNoallocMaxN; ++j) {
                        if (j >= n) break;
                        const double2 v = d[j];
                        cmul(xr, xi, __dadd_rn(cr[j], v.x), __dadd_rn(ci[j], v.y));
                    }
                    const uint32_t gt = static_cast<uint32_t>(t) ^ (static_cast<uint32_t>(t) >> 1);
                    const double w = (__popc(gt) & 1) ? -1.0 : 1.0;
                    ar = __fma_rn(w, xr, ar);
                    ai = __fma_rn(w, xi, ai);
                }
                sr = dd_add(sr, dd_mul_d(ddv{ar, 0.0}, wout));
                si = dd_add(si, dd_mul_d(ddv{ai, 0.0}, wout));
                if (seg + 1 < my_R) {
                    // next outer position: bit ctz(r+1) of the Gray code flips
                    const int64_t rn = r0 + seg + 1;
                    const int o = __ffsll(static_cast<long long>(rn)) - 1;
                    const uint64_t gn = static_cast<uint64_t>(rn) ^ (static_cast<uint64_t>(rn) >> 1);
                    const double f = ((gn >> o) & 1) ? -2.0 : 2.0;  // 0 -> 1 subtracts 2a
                    const double2 *row = a + static_cast<int64_t>(1 + p.K + o) * n;
#pragma unroll
                    for (int j = 0; j < kNoallocMaxN; ++j) {
                        if (j >= n) break;
                        const double2 v = row[j];
                        cr[j] = __fma_rn(f, v.x, cr[j]);
                        ci[j] = __fma_rn(f, v.y, ci[j]);
                    }
                    wout = -wout;
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            sr = dd_add(sr, dd_shfl_down(sr, off));
            si = dd_add(si, dd_shfl_down(si, off));
        }
        if (lane == 0) store_partial(partials, item, sr, si);
    }
}

// One block: double-double sum of the item partials, times 2^-(n-1).
__global__ void unit_finish(UnitPlan p, const unsigned char *__restrict__ scratch, double *__restrict__ out) {
    __shared__ ddv part[2 * 32];
    const double *partials = reinterpret_cast<const double *>(scratch + p.off_partials);
    ddv r{0.0, 0.0}, i{0.0, 0.0};
    for (int64_t it = threadIdx.x; it < p.items; it += blockDim.x) {
        ddv a, b;
        load_partial(partials, it, a, b);
        r = dd_add(r, a);
        i = dd_add(i, b);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        r = dd_add(r, dd_shfl_down(r, off));
        i = dd_add(i, dd_shfl_down(i, off));
    }
    if (lane == 0) {
        part[2 * warp] = r;
        part[2 * warp + 1] = i;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        r = lane < nw ? part[2 * lane] : ddv{0.0, 0.0};
        i = lane < nw ? part[2 * lane + 1] : ddv{0.0, 0.0};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            r = dd_add(r, dd_shfl_down(r, off));
            i = dd_add(i, dd_shfl_down(i, off));
        }
        if (lane == 0) {
            out[0] = ldexp(r.hi, -(p.n - 1));
            out[1] = ldexp(i.hi, -(p.n - 1));
        }
    }
}

// Per-device state, looked up once per device with that device current: the
// scratch's device address (cudaGetSymbolAddress; the array's host-side name
// is not a device address) and the SM count the split and the grid are sized
// for.
struct DeviceScratch {
    void *ptr = nullptr;
    int num_sms = 0;
};
std::mutex g_scratch_mu;
DeviceScratch g_scratch[64];

cudaError_t scratch_for_device(DeviceScratch *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    DeviceScratch &d = g_scratch[dev];
    if (!d.ptr) {
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        d.num_sms = sms > 0 ? sms : 1;
        d.ptr = p;
    }
    *out = d;
    return cudaSuccess;
}

int noalloc_fail(int code, const char *msg, cudaError_t e = cudaSuccess) {
    char buf[256];
    if (e != cudaSuccess)
        snprintf(buf, sizeof(buf), "%s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(buf, sizeof(buf), "%s", msg);
    set_last_error(buf);
    return code;
}

}  // namespace
}  // namespace pqg

using namespace pqg;

extern "C" {

// A function-try-block like every other entry point: no C++ exception (the
// mutex, the error message) crosses the C ABI.
int pqg_permanent_unit_c128_noalloc(const double *d_matrix, int64_t n, double *d_out, void *stream) try {
    if (!d_matrix || !d_out) return noalloc_fail(PQG_ERR_INVALID, "null device pointer");
    if (n < 1 || n > kNoallocMaxN)
        return noalloc_fail(PQG_ERR_TOO_LARGE, "matrix order must be between 1 and PQG_NOALLOC_MAX_N (32)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceScratch dev{};
    cudaError_t e = scratch_for_device(&dev);
    if (e != cudaSuccess) return noalloc_fail(PQG_ERR_CUDA, "scratch address", e);
    void *scratch = dev.ptr;

    // implicit plan: up to 256 inner codes, up to 64 outer positions per lane,
    // at least ~16 warps of work per SM sub-partition when the space allows
    UnitPlan p{};
    p.n = static_cast<int>(n);
    const int digits = p.n - 1;
    p.K = digits < 8 ? digits : 8;
    p.n_outer = digits - p.K;
    const int64_t Q = int64_t(1) << p.n_outer;
    int64_t R = Q / (int64_t(32) * 4 * dev.num_sms * 16);
    R = R < 1 ? 1 : (R > 64 ? 64 : R);
    p.R = static_cast<int>(R);
    const int64_t lanes = (Q + R - 1) / R;
    p.items = (lanes + 31) / 32;
    p.off_delta = 256;  // bytes [0, 256): the work-queue head
    const int64_t delta_bytes = (int64_t(1) << p.K) * p.n * 16;
    p.off_partials = p.off_delta + ((delta_bytes + 255) / 256) * 256;
    const int64_t need = p.off_partials + p.items * 32;
    if (need > static_cast<int64_t>(kScratchBytes))
        return noalloc_fail(PQG_ERR_TOO_LARGE, "problem needs more than PQG_NOALLOC_SCRATCH_BYTES of scratch");

    unsigned char *sc = static_cast<unsigned char *>(scratch);
    // the scratch keeps the last call's contents: only the queue head must start at zero
    e = cudaMemsetAsync(sc, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return noalloc_fail(PQG_ERR_CUDA, "queue reset", e);
    const double2 *a = reinterpret_cast<const double2 *>(d_matrix);
    unit_build_delta<<<64, 256, 0, s>>>(a, p, sc);
    unit_walk<<<dev.num_sms * 4, PQG_WALK_THREADS, 0, s>>>(a, p, sc);
    unit_finish<<<1, 1024, 0, s>>>(p, sc, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(PQG_ERR_CUDA, "launch", e);
    return PQG_OK;
} catch (...) {
    try {
        set_last_error("host-side failure");
    } catch (...) {
    }
    return PQG_ERR_HOST;
}

}  // extern "C"
