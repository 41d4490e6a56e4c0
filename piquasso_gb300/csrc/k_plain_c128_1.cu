// Walk-kernel instantiations, column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c128_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 17>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 18>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 19>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 20>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 21>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 22>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 23>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 24>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 25>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 26>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 27>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 28>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 29>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 30>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 31>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 32>), 0},
};

}  // namespace pqg
