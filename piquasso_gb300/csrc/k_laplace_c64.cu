// Instantiations of walk_laplace_c64 for every column count 1..32 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c64[PQG_MAX_COLS + 1] = {
    {nullptr, 0},
    {reinterpret_cast<const void *>(&walk_laplace_c64<1>), LaplaceC64Cfg<1>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<2>), LaplaceC64Cfg<2>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<3>), LaplaceC64Cfg<3>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<4>), LaplaceC64Cfg<4>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<5>), LaplaceC64Cfg<5>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<6>), LaplaceC64Cfg<6>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<7>), LaplaceC64Cfg<7>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<8>), LaplaceC64Cfg<8>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<9>), LaplaceC64Cfg<9>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<10>), LaplaceC64Cfg<10>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<11>), LaplaceC64Cfg<11>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<12>), LaplaceC64Cfg<12>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<13>), LaplaceC64Cfg<13>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<14>), LaplaceC64Cfg<14>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<15>), LaplaceC64Cfg<15>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<16>), LaplaceC64Cfg<16>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<17>), LaplaceC64Cfg<17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<18>), LaplaceC64Cfg<18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<19>), LaplaceC64Cfg<19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<20>), LaplaceC64Cfg<20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<21>), LaplaceC64Cfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<22>), LaplaceC64Cfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<23>), LaplaceC64Cfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<24>), LaplaceC64Cfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<25>), LaplaceC64Cfg<25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<26>), LaplaceC64Cfg<26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<27>), LaplaceC64Cfg<27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<28>), LaplaceC64Cfg<28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<29>), LaplaceC64Cfg<29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<30>), LaplaceC64Cfg<30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<31>), LaplaceC64Cfg<31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<32>), LaplaceC64Cfg<32>::smem_bytes},
};

}  // namespace pqg
