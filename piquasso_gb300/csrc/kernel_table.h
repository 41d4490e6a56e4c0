// Kernel tables: one walk-kernel instantiation per exact column count.
#pragma once
#include <stddef.h>

#include "pqg_plan.h"

namespace pqg {

struct KernelInfo {
    const void *fn;     // __global__ entry (launched with cudaLaunchKernel)
    size_t smem_bytes;  // dynamic shared memory per block
};

extern const KernelInfo k_plain_c128[PQG_MAX_COLS + 1];
extern const KernelInfo k_plain_c64[PQG_MAX_COLS + 1];
extern const KernelInfo k_laplace_c128[PQG_MAX_COLS + 1];
extern const KernelInfo k_laplace_c64[PQG_MAX_COLS + 1];

}  // namespace pqg
