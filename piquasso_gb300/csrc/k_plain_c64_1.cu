// Walk-kernel instantiations, column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 17>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 18>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 19>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 20>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 21>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 22>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 23>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 24>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 25>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 26>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 27>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 28>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 29>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 30>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 31>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 32>), 0},
};

}  // namespace pqg
