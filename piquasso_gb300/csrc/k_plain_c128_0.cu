// Walk-kernel instantiations, column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c128_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 1, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 2, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 3, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 4, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 5, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 6, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 7, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 8, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 9, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 10, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 11, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 12, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 13, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 14, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 15, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 16, false>), 0},
};

}  // namespace pqg
