// Walk-kernel instantiations, column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 17, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 18, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 19, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 20, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 21, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 22, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 23, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 24, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 25, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 26, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 27, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 28, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 29, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 30, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 31, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArF32, 32, false>), 0},
};

}  // namespace pqg
