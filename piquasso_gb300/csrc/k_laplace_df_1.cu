// Walk-kernel instantiations (double-float Laplace, any column multiplicities), column counts 17..32 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_df_1[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_df<17, false>), LaplaceDfCfg<17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<18, false>), LaplaceDfCfg<18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<19, false>), LaplaceDfCfg<19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<20, false>), LaplaceDfCfg<20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<21, false>), LaplaceDfCfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<22, false>), LaplaceDfCfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<23, false>), LaplaceDfCfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<24, false>), LaplaceDfCfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<25, false>), LaplaceDfCfg<25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<26, false>), LaplaceDfCfg<26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<27, false>), LaplaceDfCfg<27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<28, false>), LaplaceDfCfg<28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<29, false>), LaplaceDfCfg<29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<30, false>), LaplaceDfCfg<30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<31, false>), LaplaceDfCfg<31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_df<32, false>), LaplaceDfCfg<32>::smem_bytes},
};

}  // namespace pqg
