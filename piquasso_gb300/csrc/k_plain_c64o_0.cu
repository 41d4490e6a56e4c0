// Walk-kernel instantiations (all-ones columns), column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64o_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 1, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 2, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 3, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 4, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 5, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 6, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 7, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 8, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 9, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 10, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 11, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 12, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 13, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 14, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 15, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 16, true>), 0},
};

}  // namespace pqg
