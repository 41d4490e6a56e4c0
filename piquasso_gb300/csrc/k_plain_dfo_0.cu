// Walk-kernel instantiations (all-ones columns), column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_dfo_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 1, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 2, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 3, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 4, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 5, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 6, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 7, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 8, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 9, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 10, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 11, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 12, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 13, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 14, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 15, true>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 16, true>), 0},
};

}  // namespace pqg
