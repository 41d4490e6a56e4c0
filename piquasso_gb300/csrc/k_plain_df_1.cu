// Walk-kernel instantiations (double-float; 21..24 columns keep their seeds in shared memory, four blocks per SM), column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_df_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 17, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 18, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 19, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 20, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain_dfs<21, false>), PlainDfsCfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain_dfs<22, false>), PlainDfsCfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain_dfs<23, false>), PlainDfsCfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain_dfs<24, false>), PlainDfsCfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 25, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 26, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 27, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 28, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 29, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 30, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 31, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 32, false>), 0},
};

}  // namespace pqg
