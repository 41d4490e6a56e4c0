// Kernel tables: one walk-kernel instantiation per exact column count,
// compiled in two halves per arithmetic (k_<form>_<prec>_0.cu: 1..16,
// k_<form>_<prec>_1.cu: 17..32) so that the build runs in parallel.
#pragma once
#include <stddef.h>

#include "pqg_plan.h"

namespace pqg {

struct KernelInfo {
    const void *fn;     // __global__ entry (launched with cudaLaunchKernel)
    size_t smem_bytes;  // dynamic shared memory per block
};

extern const KernelInfo k_plain_c128_0[16];
extern const KernelInfo k_plain_c128_1[16];
extern const KernelInfo k_plain_c64_0[16];
extern const KernelInfo k_plain_c64_1[16];
extern const KernelInfo k_plain_df_0[16];
extern const KernelInfo k_plain_df_1[16];
extern const KernelInfo k_plain_c128o_0[16];  // every column of multiplicity 1
extern const KernelInfo k_plain_c128o_1[16];
extern const KernelInfo k_plain_c64o_0[16];
extern const KernelInfo k_plain_c64o_1[16];
extern const KernelInfo k_plain_dfo_0[16];
extern const KernelInfo k_plain_dfo_1[16];
extern const KernelInfo k_laplace_c128_0[16];
extern const KernelInfo k_laplace_c128_1[16];
extern const KernelInfo k_laplace_c64_0[16];
extern const KernelInfo k_laplace_c64_1[16];
extern const KernelInfo k_laplace_c64o_0[16];  // unit columns, code pairs (2..24 columns)
extern const KernelInfo k_laplace_c64o_1[16];
extern const KernelInfo k_laplace_dfo_0[16];  // double-float, every column of multiplicity 1
extern const KernelInfo k_laplace_dfo_1[16];
extern const KernelInfo k_laplace_df_0[16];  // double-float, any column multiplicities
extern const KernelInfo k_laplace_df_1[16];

// the instantiation for exactly nc columns (1 <= nc <= 32)
inline const KernelInfo &kernel_for(const KernelInfo *lo_half, const KernelInfo *hi_half, int nc) {
    return nc <= 16 ? lo_half[nc - 1] : hi_half[nc - 17];
}

}  // namespace pqg
