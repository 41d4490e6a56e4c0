// Walk-kernel instantiations of the complex64 Laplace walk for unit columns
// (two inner codes per iteration from a code-pair table), column counts
// 1..16 (generated list).  The planner selects this table for unit-column
// plans of 2..PQG_PAIRS_MAX_NC (24) columns only; the other slots hold the
// general kernel.
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c64o_0[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_c64<1, false>), LaplaceC64Cfg<1>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64p<2>), LaplaceC64PCfg<2>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<3>), LaplaceC64PCfg<3>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<4>), LaplaceC64PCfg<4>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<5>), LaplaceC64PCfg<5>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<6>), LaplaceC64PCfg<6>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<7>), LaplaceC64PCfg<7>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<8>), LaplaceC64PCfg<8>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<9>), LaplaceC64PCfg<9>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<10>), LaplaceC64PCfg<10>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<11>), LaplaceC64PCfg<11>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<12>), LaplaceC64PCfg<12>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<13>), LaplaceC64PCfg<13>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<14>), LaplaceC64PCfg<14>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<15>), LaplaceC64PCfg<15>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<16>), LaplaceC64PCfg<16>::smem_bytes},
};

}  // namespace pqg
