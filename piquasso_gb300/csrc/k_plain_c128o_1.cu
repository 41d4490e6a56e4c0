// Walk-kernel instantiations (all-ones columns), column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c128o_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 17, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 18, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 19, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 20, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 21, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 22, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 23, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 24, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 25, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 26, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 27, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 28, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 29, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 30, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 31, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 32, true>), 0},
};

}  // namespace pqg
