// Walk-kernel instantiations of the complex64 Laplace walk for unit columns
// (two inner codes per iteration from a code-pair table), column counts
// 17..32 (generated list).  The planner selects this table for unit-column
// plans of 2..PQG_PAIRS_MAX_NC (24) columns only; the other slots hold the
// general kernel.
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c64o_1[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_c64p<17>), LaplaceC64PCfg<17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<18>), LaplaceC64PCfg<18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<19>), LaplaceC64PCfg<19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<20>), LaplaceC64PCfg<20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<21>), LaplaceC64PCfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<22>), LaplaceC64PCfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<23>), LaplaceC64PCfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64p<24>), LaplaceC64PCfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<25, false>), LaplaceC64Cfg<25>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64<26, false>), LaplaceC64Cfg<26>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64<27, false>), LaplaceC64Cfg<27>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64<28, false>), LaplaceC64Cfg<28>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64<29, false>), LaplaceC64Cfg<29>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64<30, false>), LaplaceC64Cfg<30>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64<31, false>), LaplaceC64Cfg<31>::smem_bytes},  // never selected
    {reinterpret_cast<const void *>(&walk_laplace_c64<32, false>), LaplaceC64Cfg<32>::smem_bytes},  // never selected
};

}  // namespace pqg
