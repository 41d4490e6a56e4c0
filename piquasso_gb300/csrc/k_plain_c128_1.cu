// Walk-kernel instantiations, column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c128_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 17, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 18, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 19, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 20, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 21, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 22, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 23, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 24, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 25, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 26, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 27, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 28, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 29, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 30, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 31, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF64, 32, false>), 0},
};

}  // namespace pqg
