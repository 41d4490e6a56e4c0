// Walk-kernel instantiations (double-float; 21..24 columns keep their seeds in shared memory, four blocks per SM) (all-ones columns), column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_dfo_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 17, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 18, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 19, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 20, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain_dfs<21, true>), PlainDfsCfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain_dfs<22, true>), PlainDfsCfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain_dfs<23, true>), PlainDfsCfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain_dfs<24, true>), PlainDfsCfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 25, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 26, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 27, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 28, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 29, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 30, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 31, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 32, true>), 0},
};

}  // namespace pqg
