// Walk-kernel instantiations (double-float Laplace, any column multiplicities), column counts 1..16 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_df_0[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_df<1, false>), LaplaceDfCfg<1>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<2, false>), LaplaceDfCfg<2>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<3, false>), LaplaceDfCfg<3>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<4, false>), LaplaceDfCfg<4>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<5, false>), LaplaceDfCfg<5>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<6, false>), LaplaceDfCfg<6>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<7, false>), LaplaceDfCfg<7>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<8, false>), LaplaceDfCfg<8>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<9, false>), LaplaceDfCfg<9>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<10, false>), LaplaceDfCfg<10>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<11, false>), LaplaceDfCfg<11>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<12, false>), LaplaceDfCfg<12>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<13, false>), LaplaceDfCfg<13>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<14, false>), LaplaceDfCfg<14>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<15, false>), LaplaceDfCfg<15>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<16, false>), LaplaceDfCfg<16>::smem_bytes},
};

}  // namespace pqg
