// Walk-kernel instantiations, column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 1>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 2>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 3>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 4>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 5>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 6>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 7>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 8>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 9>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 10>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 11>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 12>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 13>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 14>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 15>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 16>), 0},
};

}  // namespace pqg
