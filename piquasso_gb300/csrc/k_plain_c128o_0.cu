// Walk-kernel instantiations (all-ones columns), column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c128o_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 1, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 2, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 3, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 4, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 5, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 6, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 7, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 8, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 9, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 10, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 11, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 12, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 13, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 14, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 15, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 16, true>), 0},
};

}  // namespace pqg
