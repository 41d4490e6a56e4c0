// Instantiations of walk_plain_c128 for every column count 1..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c128[PQG_MAX_COLS + 1] = {
    {nullptr, 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<1>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<2>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<3>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<4>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<5>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<6>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<7>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<8>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<9>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<10>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<11>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<12>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<13>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<14>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<15>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<16>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<17>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<18>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<19>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<20>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<21>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<22>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<23>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<24>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<25>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<26>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<27>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<28>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<29>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<30>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<31>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c128<32>), 0},
};

}  // namespace pqg
