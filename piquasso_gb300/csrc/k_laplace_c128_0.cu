// Walk-kernel instantiations, column counts 1..16 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c128_0[16] = {
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
};

}  // namespace pqg
