// Walk-kernel instantiations (all-ones columns), column counts 17..32 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c64o_1[16] = {
    {reinterpret_cast<const void *>(&walk_laplace_c64<17, true>), LaplaceC64Cfg<17>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<18, true>), LaplaceC64Cfg<18>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<19, true>), LaplaceC64Cfg<19>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<20, true>), LaplaceC64Cfg<20>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<21, true>), LaplaceC64Cfg<21>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<22, true>), LaplaceC64Cfg<22>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<23, true>), LaplaceC64Cfg<23>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<24, true>), LaplaceC64Cfg<24>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<25, true>), LaplaceC64Cfg<25>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<26, true>), LaplaceC64Cfg<26>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<27, true>), LaplaceC64Cfg<27>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<28, true>), LaplaceC64Cfg<28>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<29, true>), LaplaceC64Cfg<29>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<30, true>), LaplaceC64Cfg<30>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<31, true>), LaplaceC64Cfg<31>::smem_bytes},
    {reinterpret_cast<const void *>(&walk_laplace_c64<32, true>), LaplaceC64Cfg<32>::smem_bytes},
};

}  // namespace pqg
