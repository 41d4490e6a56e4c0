// Walk-kernel instantiations (double-float Laplace, all-ones columns), column counts 1..16 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_dfo_0[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_df<1, true>), LaplaceDfCfg<1>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<2, true>), LaplaceDfCfg<2>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<3, true>), LaplaceDfCfg<3>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<4, true>), LaplaceDfCfg<4>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<5, true>), LaplaceDfCfg<5>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<6, true>), LaplaceDfCfg<6>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<7, true>), LaplaceDfCfg<7>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<8, true>), LaplaceDfCfg<8>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<9, true>), LaplaceDfCfg<9>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<10, true>), LaplaceDfCfg<10>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<11, true>), LaplaceDfCfg<11>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<12, true>), LaplaceDfCfg<12>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<13, true>), LaplaceDfCfg<13>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<14, true>), LaplaceDfCfg<14>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<15, true>), LaplaceDfCfg<15>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<16, true>), LaplaceDfCfg<16>::smem_bytes},
};

}  // namespace pqg
