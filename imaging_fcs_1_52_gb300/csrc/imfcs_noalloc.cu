// imfcs_noalloc.cu -- batched LM fit on device buffers that allocates nothing.
//
// Same fit as imfcs_fit (Gpufit semantics, lm_kernel) but every argument is a
// device pointer and the per-fit scratch (parameters in internal units, the
// model constants, the fitted parameters) lives in a file-scope __device__
// array of fixed size.  The array's device address is looked up on every call
// with cudaGetSymbolAddress in the caller's current context (a symbol's
// address belongs to a context, so a cached address would go stale after a
// cudaDeviceReset or in another context on the same device); the lookup
// allocates nothing.  The call issues no cudaMalloc / cudaFree and no
// allocating library routine.
#include "imfcs_args.h"
#include "imfcs_host.h"

namespace imfcs {

cudaError_t launch_lm(const FitArgs &a, int num_sms, cudaStream_t stream);

// Per fit: init (11) + constants (9) + fitted parameters (11) floats.
constexpr int kNoAllocPerFit = IMFCS_NPARAM + IMFCS_NCONST + IMFCS_NPARAM;
static __device__ __align__(256) float g_noalloc_scratch[(size_t)IMFCS_FIT_NOALLOC_MAX_FITS * kNoAllocPerFit];

// Internal-unit initial values and per-fit constants from the caller's
// [fit][nparam] array (ACF_1D: SI units, constants at 11..19).
__global__ void noalloc_prepare_kernel(int nfits, int nparam, int np, int acf, const float *init_si,
                                       float *init_int, float *cst)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfits) return;
    const float *src = init_si + (size_t)f * nparam;
    for (int i = 0; i < np; i++)
        init_int[(size_t)f * IMFCS_NPARAM + i] = acf ? (float)((double)src[i] / param_unit(i)) : src[i];
    if (acf)
        for (int i = 0; i < IMFCS_NCONST; i++) cst[(size_t)f * IMFCS_NCONST + i] = src[IMFCS_NPARAM + i];
}

// Fitted parameters back to the caller's layout: fitted values in SI units,
// every other entry copied from the initial array.
__global__ void noalloc_finish_kernel(int nfits, int nparam, int np, int acf, const float *init_si,
                                      const float *par_int, float *out)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfits) return;
    for (int i = 0; i < nparam; i++) {
        float v = init_si[(size_t)f * nparam + i];
        if (i < np) {
            const float p = par_int[(size_t)f * IMFCS_NPARAM + i];
            v = acf ? (float)((double)p * param_unit(i)) : p;
        }
        out[(size_t)f * nparam + i] = v;
    }
}

}  // namespace imfcs

using namespace imfcs;

extern "C" int imfcs_fit_device_noalloc(int n_fits, int n_points, const float *data, const float *weights,
                                        int model_id, const float *initial_parameters, float tolerance,
                                        int max_n_iterations, int num_valid_coefs,
                                        const int *parameters_to_fit, const float *user_info,
                                        float *output_parameters, int *output_states,
                                        float *output_chi_squares, int *output_n_iterations, void *stream)
{
    if (n_fits < 0 || n_points <= 0 || !data || !initial_parameters || !parameters_to_fit || !user_info ||
        !output_parameters) {
        set_error("invalid argument");
        return -1;
    }
    if (n_fits > IMFCS_FIT_NOALLOC_MAX_FITS) {
        set_error("imfcs_fit_device_noalloc: n_fits exceeds IMFCS_FIT_NOALLOC_MAX_FITS (16384); split the batch");
        return -1;
    }
    if (model_id != IMFCS_MODEL_ACF_1D && model_id != IMFCS_MODEL_LINEAR_1D) {
        set_error("unsupported model id");
        return -1;
    }
    const bool acf = model_id == IMFCS_MODEL_ACF_1D;
    const int nparam = acf ? IMFCS_ACF_1D_NPARAM : IMFCS_LINEAR_1D_NPARAM;
    const int np = acf ? IMFCS_NPARAM : num_valid_coefs;
    if (!acf && (num_valid_coefs < 1 || num_valid_coefs > IMFCS_LINEAR_1D_NPARAM)) {
        set_error("num_valid_coefs out of range");
        return -1;
    }
    if (n_fits == 0) return 0;
    // Errors left on this thread by earlier, unrelated work are reported as
    // such instead of being attributed to the launches below.
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(cuda_msg(e, "error pending before imfcs_fit_device_noalloc")); return -1; }
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "cudaGetDevice")); return -1; }
    // the scratch array's address in the current context, and the SM count
    float *scratch = nullptr;
    e = cudaGetSymbolAddress((void **)&scratch, g_noalloc_scratch);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "cudaGetSymbolAddress(scratch)")); return -1; }
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "cudaDeviceGetAttribute(SM count)")); return -1; }
    cudaStream_t s = (cudaStream_t)stream;
    float *init_int = scratch;
    float *cst = init_int + (size_t)IMFCS_FIT_NOALLOC_MAX_FITS * IMFCS_NPARAM;
    float *par = cst + (size_t)IMFCS_FIT_NOALLOC_MAX_FITS * IMFCS_NCONST;

    const int threads = 128, blocks = (n_fits + threads - 1) / threads;
    noalloc_prepare_kernel<<<blocks, threads, 0, s>>>(n_fits, nparam, np, acf, initial_parameters, init_int, cst);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(cuda_msg(e, "noalloc prepare")); return -1; }

    FitArgs a;
    memset(&a, 0, sizeof(a));
    a.nfits = n_fits;
    a.npts = n_points;
    a.model = model_id;
    a.np = np;
    for (int i = 0; i < np; i++)
        if (parameters_to_fit[i]) a.idx[a.k++] = i;
    a.max_iter = max_n_iterations > 0 ? max_n_iterations : 1;
    a.tol = tolerance > 0.f ? tolerance : 1e-30f;
    a.y = data;
    a.w = weights;
    a.x = user_info;
    a.init = init_int;
    a.init_stride = IMFCS_NPARAM;
    a.cst = acf ? cst : nullptr;
    a.out_par = par;
    a.out_stride = IMFCS_NPARAM;
    a.out_chi2 = output_chi_squares;
    a.out_state = output_states;
    a.out_iter = output_n_iterations;
    e = launch_lm(a, sms, s);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "lm_kernel")); return -1; }

    noalloc_finish_kernel<<<blocks, threads, 0, s>>>(n_fits, nparam, np, acf, initial_parameters, par,
                                                     output_parameters);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(cuda_msg(e, "noalloc finish")); return -1; }
    return 0;
}
