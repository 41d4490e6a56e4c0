// Walk-kernel instantiations, column counts 1..16 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_df_0[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 1, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 2, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 3, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 4, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 5, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 6, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 7, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 8, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 9, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 10, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 11, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 12, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 13, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 14, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 15, false>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 16, false>), 0},
};

}  // namespace pqg
