// Walk-kernel instantiations (double-float Laplace, all-ones columns), column counts 1..16 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_dfo_0[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_df<1>), LaplaceDfCfg<1>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<2>), LaplaceDfCfg<2>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<3>), LaplaceDfCfg<3>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<4>), LaplaceDfCfg<4>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<5>), LaplaceDfCfg<5>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<6>), LaplaceDfCfg<6>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<7>), LaplaceDfCfg<7>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<8>), LaplaceDfCfg<8>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<9>), LaplaceDfCfg<9>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<10>), LaplaceDfCfg<10>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<11>), LaplaceDfCfg<11>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<12>), LaplaceDfCfg<12>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<13>), LaplaceDfCfg<13>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<14>), LaplaceDfCfg<14>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<15>), LaplaceDfCfg<15>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<16>), LaplaceDfCfg<16>::smem_bytes},
};

}  // namespace pqg
