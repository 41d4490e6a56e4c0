// Walk-kernel instantiations, column counts 17..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_df_1[16] = {
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 17>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 18>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 19>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 20>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 21>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 22>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 23>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 24>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 25>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 26>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 27>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 28>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 29>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 30>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 31>), 0},
    {reinterpret_cast<const void *>(&walk_plain<ArDF, 32>), 0},
};

}  // namespace pqg
