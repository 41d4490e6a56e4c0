// Walk-kernel instantiations (all-ones columns), column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64o_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 17, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 18, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 19, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 20, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 21, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 22, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 23, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 24, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 25, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 26, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 27, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 28, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 29, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 30, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 31, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 32, true>), 0},
};

}  // namespace pqg
