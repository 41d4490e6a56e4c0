// Walk-kernel instantiations, column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 1, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 2, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 3, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 4, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 5, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 6, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 7, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 8, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 9, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 10, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 11, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 12, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 13, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 14, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 15, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 16, false>), 0},
};

}  // namespace pqg
