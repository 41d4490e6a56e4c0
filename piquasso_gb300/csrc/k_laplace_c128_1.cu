// Walk-kernel instantiations, column counts 17..32 (generated list).
#include "walk_laplace.cuh"
#include "kernel_table.h"

namespace pqg {

const KernelInfo k_laplace_c128_1[16] = {
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
