// Instantiations of walk_plain_c64 for every column count 1..32 (generated list).
#include "walk_plain.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_plain_c64[PQG_MAX_COLS + 1] = {
    {nullptr, 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<1>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<2>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<3>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<4>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<5>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<6>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<7>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<8>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<9>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<10>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<11>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<12>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<13>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<14>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<15>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<16>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<17>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<18>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<19>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<20>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<21>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<22>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<23>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<24>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<25>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<26>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<27>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<28>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<29>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<30>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<31>), 0},
    {reinterpret_cast<const void *>(&walk_plain_c64<32>), 0},
};

}  // namespace pqg
