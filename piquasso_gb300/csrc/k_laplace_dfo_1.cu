// Walk-kernel instantiations (double-float Laplace, all-ones columns), column counts 17..32 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_dfo_1[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_df<17>), LaplaceDfCfg<17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<18>), LaplaceDfCfg<18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<19>), LaplaceDfCfg<19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<20>), LaplaceDfCfg<20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<21>), LaplaceDfCfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<22>), LaplaceDfCfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<23>), LaplaceDfCfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<24>), LaplaceDfCfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<25>), LaplaceDfCfg<25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<26>), LaplaceDfCfg<26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<27>), LaplaceDfCfg<27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<28>), LaplaceDfCfg<28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<29>), LaplaceDfCfg<29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<30>), LaplaceDfCfg<30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<31>), LaplaceDfCfg<31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<32>), LaplaceDfCfg<32>::smem_bytes},
};

}  // namespace pqg
