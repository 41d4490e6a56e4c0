// Walk-kernel instantiations, column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c128_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 1>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 2>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 3>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 4>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 5>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 6>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 7>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 8>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 9>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 10>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 11>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 12>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 13>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 14>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 15>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 16>), 0},
};

}  // namespace pqg
