// Walk-kernel instantiations, column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 17, false>), PlainCfg<ArF32, 17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 18, false>), PlainCfg<ArF32, 18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 19, false>), PlainCfg<ArF32, 19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 20, false>), PlainCfg<ArF32, 20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 21, false>), PlainCfg<ArF32, 21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 22, false>), PlainCfg<ArF32, 22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 23, false>), PlainCfg<ArF32, 23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 24, false>), PlainCfg<ArF32, 24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 25, false>), PlainCfg<ArF32, 25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 26, false>), PlainCfg<ArF32, 26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 27, false>), PlainCfg<ArF32, 27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 28, false>), PlainCfg<ArF32, 28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 29, false>), PlainCfg<ArF32, 29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 30, false>), PlainCfg<ArF32, 30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 31, false>), PlainCfg<ArF32, 31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 32, false>), PlainCfg<ArF32, 32>::smem_bytes},
};

}  // namespace pqg
