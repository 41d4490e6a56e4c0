// Instantiations of walk_laplace_c128 for every column count 1..32 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c128[PQG_MAX_COLS + 1] = {
    {nullptr, 0},
    {reinterpret_cast<const void *>(&walk_laplace_c128<1>), LaplaceC128Cfg<1>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<2>), LaplaceC128Cfg<2>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<3>), LaplaceC128Cfg<3>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<4>), LaplaceC128Cfg<4>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<5>), LaplaceC128Cfg<5>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<6>), LaplaceC128Cfg<6>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<7>), LaplaceC128Cfg<7>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<8>), LaplaceC128Cfg<8>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<9>), LaplaceC128Cfg<9>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<10>), LaplaceC128Cfg<10>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<11>), LaplaceC128Cfg<11>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<12>), LaplaceC128Cfg<12>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<13>), LaplaceC128Cfg<13>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<14>), LaplaceC128Cfg<14>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<15>), LaplaceC128Cfg<15>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<16>), LaplaceC128Cfg<16>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<17>), LaplaceC128Cfg<17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<18>), LaplaceC128Cfg<18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<19>), LaplaceC128Cfg<19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<20>), LaplaceC128Cfg<20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<21>), LaplaceC128Cfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<22>), LaplaceC128Cfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<23>), LaplaceC128Cfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<24>), LaplaceC128Cfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<25>), LaplaceC128Cfg<25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<26>), LaplaceC128Cfg<26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<27>), LaplaceC128Cfg<27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<28>), LaplaceC128Cfg<28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<29>), LaplaceC128Cfg<29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<30>), LaplaceC128Cfg<30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<31>), LaplaceC128Cfg<31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c128<32>), LaplaceC128Cfg<32>::smem_bytes},
};

}  // namespace pqg
