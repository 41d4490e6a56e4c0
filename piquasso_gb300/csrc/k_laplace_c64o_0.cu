// Walk-kernel instantiations (all-ones columns), column counts 1..16 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c64o_0[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_c64<1, true>), LaplaceC64Cfg<1>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<2, true>), LaplaceC64Cfg<2>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<3, true>), LaplaceC64Cfg<3>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<4, true>), LaplaceC64Cfg<4>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<5, true>), LaplaceC64Cfg<5>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<6, true>), LaplaceC64Cfg<6>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<7, true>), LaplaceC64Cfg<7>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<8, true>), LaplaceC64Cfg<8>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<9, true>), LaplaceC64Cfg<9>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<10, true>), LaplaceC64Cfg<10>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<11, true>), LaplaceC64Cfg<11>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<12, true>), LaplaceC64Cfg<12>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<13, true>), LaplaceC64Cfg<13>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<14, true>), LaplaceC64Cfg<14>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<15, true>), LaplaceC64Cfg<15>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<16, true>), LaplaceC64Cfg<16>::smem_bytes},
};

}  // namespace pqg
