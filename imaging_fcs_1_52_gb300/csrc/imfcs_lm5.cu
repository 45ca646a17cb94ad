// imfcs_lm5.cu -- lm_kernel for up to 5 free parameters and its launcher
// (a translation unit of its own so that the unrolled variants compile in
// parallel; kernel stubs of templates do not link across units).
#include "imfcs_lm.cuh"

namespace imfcs {

cudaError_t launch_lm_k5(const FitArgs &a, bool big, int blocks, int threads, size_t smem, cudaStream_t s)
{
    void (*kern)(FitArgs) = big ? lm_kernel<5, true> : lm_kernel<5, false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, threads, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace imfcs
