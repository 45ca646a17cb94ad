// imfcs_tma.cuh -- TMA (cp.async.bulk.tensor) staging and mbarrier helpers
// shared by the streaming kernels, plus the host-side tensor-map encoder.
//
// Every wait is bounded: mbar_wait gives up after ~1 s of polling and
// returns false; callers record an error flag and leave their loops (after
// waiting, again bounded, for their own copies still in flight).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdint.h>

namespace imfcs {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One 3-D box load [t][y][x] into shared memory, completing on `mbar`
// (which also receives the expected byte count from this thread's arrival).
__device__ __forceinline__ void tma_load_box(const CUtensorMap *tmap, void *dst, uint64_t *mbar, int x, int y,
                                             int t, uint32_t bytes)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(t), "r"(smem_u32(mbar))
        : "memory");
}

// Bounded wait on an mbarrier phase.  Returns false after ~1 s.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity)
{
    const uint32_t a = smem_u32(mbar);
    for (int i = 0; i < (1 << 20); i++) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(1000)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Host: cuTensorMapEncodeTiled from the driver (resolved once).
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            return nullptr;
        fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

}  // namespace imfcs
