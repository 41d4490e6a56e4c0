// Walk-kernel instantiations (all-ones columns), column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64o_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 17, true>), PlainCfg<ArF32, 17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 18, true>), PlainCfg<ArF32, 18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 19, true>), PlainCfg<ArF32, 19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 20, true>), PlainCfg<ArF32, 20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 21, true>), PlainCfg<ArF32, 21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 22, true>), PlainCfg<ArF32, 22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 23, true>), PlainCfg<ArF32, 23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 24, true>), PlainCfg<ArF32, 24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 25, true>), PlainCfg<ArF32, 25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 26, true>), PlainCfg<ArF32, 26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 27, true>), PlainCfg<ArF32, 27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 28, true>), PlainCfg<ArF32, 28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 29, true>), PlainCfg<ArF32, 29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 30, true>), PlainCfg<ArF32, 30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 31, true>), PlainCfg<ArF32, 31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 32, true>), PlainCfg<ArF32, 32>::smem_bytes},
};

}  // namespace pqg
