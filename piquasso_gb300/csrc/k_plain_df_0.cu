// Walk-kernel instantiations, column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_df_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 1>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 2>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 3>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 4>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 5>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 6>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 7>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 8>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 9>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 10>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 11>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 12>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 13>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 14>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 15>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 16>), 0},
};

}  // namespace pqg
