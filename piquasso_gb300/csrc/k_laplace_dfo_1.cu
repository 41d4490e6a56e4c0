// Walk-kernel instantiations (double-float Laplace, all-ones columns), column counts 17..32 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_dfo_1[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_df<17, true>), LaplaceDfCfg<17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<18, true>), LaplaceDfCfg<18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<19, true>), LaplaceDfCfg<19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<20, true>), LaplaceDfCfg<20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<21, true>), LaplaceDfCfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<22, true>), LaplaceDfCfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<23, true>), LaplaceDfCfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<24, true>), LaplaceDfCfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<25, true>), LaplaceDfCfg<25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<26, true>), LaplaceDfCfg<26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<27, true>), LaplaceDfCfg<27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<28, true>), LaplaceDfCfg<28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<29, true>), LaplaceDfCfg<29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<30, true>), LaplaceDfCfg<30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<31, true>), LaplaceDfCfg<31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<32, true>), LaplaceDfCfg<32>::smem_bytes},
};

}  // namespace pqg
