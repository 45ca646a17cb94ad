// imfcs_mlp.cu -- the learned part: a small MLP surrogate that maps a
// normalised ACF and its standard deviation to initial fit parameters, with
// BF16 tensor-core forward and backward kernels (FP32 accumulation), Adam in
// FP32 master weights, and the input features built on the device from the
// correlator's outputs.  It has no counterpart in the reference, whose fits
// start from fixed values (N = 1, D = 1 um^2/s, G = 0; Imaging_FCS_1_52.java
// :1958-1970); plain LM from those values stays the fallback and the arbiter of
// the seeded fits.
//
// Network: x[128] -> z1 = x W1 + b1 [256] -> h1 = GELU(z1) -> z2 = h1 W2 + b2
// [256] -> h2 = GELU(z2) -> y = h2 W3 + b3 [4]; GELU(z) = z Phi(z) (erf
// form).  Inputs: g_i = G(lag i) / G(lag 1) and s_i = sd(lag i) / |G(lag 1)|
// for lags i = 1..64.  Outputs (standardised): log D [um^2/s], log(N G(1)),
// G_inf / G(1), the fraction of a second component.
//
// GEMMs: C[M][N] = A[M][K] B[K][N] with arbitrary element strides (so the
// transposes of the backward pass are strides, not copies), BF16 operands,
// FP32 accumulators, mma.sync.m16n8k16 on 64x64 CTA tiles (4 warps, 32x32
// each), operands staged through shared memory.  Epilogues: bias + GELU
// (keeps z in FP32 for the backward pass, h in BF16 for the next layer),
// bias, the GELU derivative (dz = acc GELU'(z), BF16), plain FP32.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cuda_bf16.h>

#include <random>
#include <vector>

#include "imfcs_gb300.h"
#include "imfcs_host.h"

namespace imfcs {

constexpr int kIn = 128, kHid = 256, kOut = 4;
constexpr int kLagsIn = 64;
constexpr size_t kW1 = (size_t)kIn * kHid, kW2 = (size_t)kHid * kHid, kW3 = (size_t)kHid * kOut;
// flat FP32 parameter vector: W1 b1 W2 b2 W3 b3
constexpr size_t kParams = kW1 + kHid + kW2 + kHid + kW3 + kOut;

enum { EPI_BIAS_GELU = 0, EPI_BIAS = 1, EPI_STORE = 2, EPI_GELU_BWD = 3 };

struct GemmArgs {
    int M, N, K;
    const __nv_bfloat16 *A;
    long lam, lak;              // A(m, k) = A[m lam + k lak]
    const __nv_bfloat16 *B;
    long lbk, lbn;              // B(k, n) = B[k lbk + n lbn]
    const float *bias;          // [N]
    const float *zin;           // EPI_GELU_BWD: z [M][N]
    float *outf;                // [M][N] FP32 (EPI_BIAS, EPI_STORE; EPI_BIAS_GELU: z)
    __nv_bfloat16 *outh;        // [M][N] BF16 (EPI_BIAS_GELU: h; EPI_GELU_BWD: dz)
    float alpha;                // EPI_STORE scale
};

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad_f(float z)
{
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * __expf(-0.5f * z * z);
}

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int kTM = 64, kTN = 64, kTK = 32, kPad = 8;

template <int EPI>
__global__ void __launch_bounds__(128) mlp_gemm_kernel(GemmArgs g)
{
    __shared__ __align__(16) __nv_bfloat16 As[kTM][kTK + kPad];   // [m][k]
    __shared__ __align__(16) __nv_bfloat16 Bs[kTN][kTK + kPad];   // [n][k]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gid = lane >> 2, tig = lane & 3;
    const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < g.K; k0 += kTK) {
        // stage the tiles (bounds-checked, zero outside); consecutive
        // threads walk the operand's unit-stride dimension
        const bool a_kfast = g.lak == 1, b_kfast = g.lbn != 1;
        for (int i = tid; i < kTM * kTK; i += 128) {
            const int r = a_kfast ? i / kTK : i % kTM, c = a_kfast ? i % kTK : i / kTM;
            const int m = m0 + r, k = k0 + c;
            As[r][c] = (m < g.M && k < g.K) ? g.A[(long)m * g.lam + (long)k * g.lak] : zero;
        }
        for (int i = tid; i < kTN * kTK; i += 128) {
            const int r = b_kfast ? i / kTK : i % kTN, c = b_kfast ? i % kTK : i / kTN;
            const int n = n0 + r, k = k0 + c;
            Bs[r][c] = (n < g.N && k < g.K) ? g.B[(long)k * g.lbk + (long)n * g.lbn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kTK; ks += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                const int r = wm + mt * 16 + gid, c = ks + 2 * tig;
                af[mt][0] = *(const uint32_t *)&As[r][c];
                af[mt][1] = *(const uint32_t *)&As[r + 8][c];
                af[mt][2] = *(const uint32_t *)&As[r][c + 8];
                af[mt][3] = *(const uint32_t *)&As[r + 8][c + 8];
            }
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const int r = wn + nt * 8 + gid, c = ks + 2 * tig;
                bf[nt][0] = *(const uint32_t *)&Bs[r][c];
                bf[nt][1] = *(const uint32_t *)&Bs[r][c + 8];
            }
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 4; nt++) mma_bf16(acc[mt][nt], af[mt], bf[nt]);
        }
        __syncthreads();
    }
    // epilogue: fragment element (row gid [+8], col 2 tig [+1])
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int m = m0 + wm + mt * 16 + gid + (e >= 2 ? 8 : 0);
                const int n = n0 + wn + nt * 8 + 2 * tig + (e & 1);
                if (m >= g.M || n >= g.N) continue;
                const size_t o = (size_t)m * g.N + n;
                const float v = acc[mt][nt][e];
                if (EPI == EPI_BIAS_GELU) {
                    const float z = v + g.bias[n];
                    g.outf[o] = z;
                    g.outh[o] = __float2bfloat16(gelu_f(z));
                } else if (EPI == EPI_BIAS) {
                    g.outf[o] = v + g.bias[n];
                } else if (EPI == EPI_STORE) {
                    g.outf[o] = g.alpha * v;
                } else {
                    g.outh[o] = __float2bfloat16(v * gelu_grad_f(g.zin[o]));
                }
            }
}

template <int EPI>
static cudaError_t gemm(const GemmArgs &g, cudaStream_t s)
{
    dim3 grid((g.N + kTN - 1) / kTN, (g.M + kTM - 1) / kTM);
    mlp_gemm_kernel<EPI><<<grid, 128, 0, s>>>(g);
    return cudaGetLastError();
}

// FP32 -> BF16 copy
__global__ void to_bf16_kernel(const float *in, __nv_bfloat16 *out, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16(in[i]);
}

// MSE loss on standardised targets and its gradient dy = 2 (y - t) / (B * 4)
// (FP32 and BF16); loss accumulates into *loss (one double).
__global__ void mse_kernel(const float *y, const float *t, int n, float *dy, __nv_bfloat16 *dyh, double *loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n * kOut) {
        const float d = y[i] - t[i];
        const float gr = 2.f * d / (float)(n * kOut);
        dy[i] = gr;
        dyh[i] = __float2bfloat16(gr);
        l = d * d;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)l / (double)(n * kOut));
}

// column sums over the batch: db[n] = sum_m d[m][n] (FP32 or BF16 input)
template <class T>
__global__ void colsum_kernel(const T *d, int M, int N, float *db)
{
    const int n = blockIdx.x;
    float s = 0.f;
    for (int m = threadIdx.x; m < M; m += blockDim.x) s += (float)d[(size_t)m * N + n];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        db[n] = t;
    }
}

// Adam on the flat FP32 parameters; refreshes the BF16 weight copies.
__global__ void adam_kernel(float *w, const float *gr, float *m, float *v, size_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = gr[i];
    const float mi = b1 * m[i] + (1.f - b1) * g, vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// Features of the surrogate from correlator outputs ([pix][chanum], FP64):
// g_i = G(i) / G(1) clamped to [-8, 8], s_i = sqrt(var(i)) / |G(1)| clamped
// to [0, 8], for i = 1..64; non-finite values (a pixel without a valid
// correlation) become 0.
__global__ void features_kernel(int npix, int chanum, const double *acf, const double *var, float *x)
{
    const int pix = blockIdx.x, i = threadIdx.x;   // 64 threads
    if (pix >= npix) return;
    const double g1 = acf[(size_t)pix * chanum + 1];
    const double ag = acf[(size_t)pix * chanum + 1 + i], vg = var[(size_t)pix * chanum + 1 + i];
    float g = (float)(ag / g1), s = (float)(sqrt(vg) / fabs(g1));
    g = isfinite(g) ? fminf(fmaxf(g, -8.f), 8.f) : 0.f;
    s = isfinite(s) ? fminf(s, 8.f) : 0.f;
    x[(size_t)pix * kIn + i] = g;
    x[(size_t)pix * kIn + kLagsIn + i] = s;
}

struct FreeIdx {
    int k, idx[IMFCS_NPARAM];
};

// Predictions -> LM initial values (internal units) per pixel: D from log D,
// N from log(N G1) / G1, G from G_inf / G1 * G1, each only where that
// parameter is free and the seed is finite (N, D also positive); every other
// parameter keeps the configured value.  Writes init[pix][11].
__global__ void seed_kernel(int npix, int chanum, FreeIdx f, const double *acf, const float *pred,
                            const float *base_init, float *init)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const double g1 = acf[(size_t)pix * chanum + 1];
    float *o = init + (size_t)pix * IMFCS_NPARAM;
    for (int i = 0; i < IMFCS_NPARAM; i++) o[i] = base_init[i];
    bool fn = false, fd = false, fg = false;
    for (int i = 0; i < f.k; i++) {
        fn |= f.idx[i] == 0;
        fd |= f.idx[i] == 1;
        fg |= f.idx[i] == 4;
    }
    const float *p = pred + (size_t)pix * kOut;
    const float d = expf(p[0]), ng = expf(p[1]);
    const float n = (float)(ng / g1), gi = (float)(p[2] * g1);
    if (fd && isfinite(d) && d > 0.f) o[1] = d;
    if (fn && isfinite(n) && n > 0.f) o[0] = n;
    if (fg && isfinite(gi)) o[4] = gi;
}

__global__ void seed_select_kernel(int npix, FreeIdx f, const float *par, const int *state, const float *chi2,
                                   const int *pstate, const float *pchi2, const float *y, const float *w, int npts,
                                   int *todo, int *counts)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const float *p = par + (size_t)pix * IMFCS_NPARAM;
    bool ok = state[pix] == IMFCS_STATE_CONVERGED && p[0] > 0.f && p[1] > 0.f;
    for (int i = 0; i < f.k; i++) ok = ok && isfinite(p[f.idx[i]]);
    bool worse = false;
    if (ok && pchi2 && pstate[pix] == IMFCS_STATE_CONVERGED) worse = !(chi2[pix] <= 1.01f * pchi2[pix]);
    // a pixel whose data hold a non-finite value fails from any start: no refit
    bool data_ok = true;
    for (int i = 0; i < npts && data_ok; i++)
        data_ok = isfinite(y[(size_t)pix * npts + i]) && (!w || isfinite(w[(size_t)pix * npts + i]));
    const int t = data_ok && (!ok || worse);
    todo[pix] = t;
    if (t) atomicAdd(&counts[0], 1);
    if (worse) atomicAdd(&counts[1], 1);
}

cudaError_t launch_seed_select(int npix, int k, const int *idx, const float *par, const int *state,
                               const float *chi2, const int *plain_state, const float *plain_chi2, const float *y,
                               const float *w, int npts, int *todo, int *counts, cudaStream_t s)
{
    FreeIdx f;
    f.k = k;
    for (int i = 0; i < IMFCS_NPARAM; i++) f.idx[i] = i < k ? idx[i] : 0;
    seed_select_kernel<<<(npix + 127) / 128, 128, 0, s>>>(npix, f, par, state, chi2, plain_state, plain_chi2, y, w,
                                                          npts, todo, counts);
    return cudaGetLastError();
}

}  // namespace imfcs

using namespace imfcs;

// ---------------------------------------------------------------------------
// Host side: the surrogate handle.
// ---------------------------------------------------------------------------
struct imfcs_surrogate {
    float *w = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;   // flat FP32 [kParams]
    __nv_bfloat16 *wh = nullptr;                                          // BF16 copy [kParams]
    float tmean[kOut] = {0, 0, 0, 0}, tstd[kOut] = {1, 1, 1, 1};
    int adam_t = 0;
    int cap = 0;                       // batch capacity of the work buffers
    __nv_bfloat16 *xh = nullptr, *h1 = nullptr, *h2 = nullptr, *dyh = nullptr, *dz2 = nullptr, *dz1 = nullptr;
    float *z1 = nullptr, *z2 = nullptr, *y = nullptr, *dy = nullptr, *tn = nullptr;
    double *loss = nullptr;
    std::vector<void *> bufs;
    ~imfcs_surrogate()
    {
        for (void *p : bufs) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T *&p, size_t n)
    {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
        if (e == cudaSuccess) { bufs.push_back(q); p = (T *)q; }
        return e;
    }
    cudaError_t reserve(int n)
    {
        if (n <= cap) return cudaSuccess;
        cudaError_t e = cudaSuccess;
        const size_t N = (size_t)n;
        if (e == cudaSuccess) e = alloc(xh, N * kIn);
        if (e == cudaSuccess) e = alloc(h1, N * kHid);
        if (e == cudaSuccess) e = alloc(h2, N * kHid);
        if (e == cudaSuccess) e = alloc(z1, N * kHid);
        if (e == cudaSuccess) e = alloc(z2, N * kHid);
        if (e == cudaSuccess) e = alloc(y, N * kOut);
        if (e == cudaSuccess) e = alloc(dy, N * kOut);
        if (e == cudaSuccess) e = alloc(dyh, N * kOut);
        if (e == cudaSuccess) e = alloc(tn, N * kOut);
        if (e == cudaSuccess) e = alloc(dz2, N * kHid);
        if (e == cudaSuccess) e = alloc(dz1, N * kHid);
        if (e == cudaSuccess) cap = n;
        return e;
    }
    // parameter blocks
    float *W1() { return w; }
    float *B1() { return w + kW1; }
    float *W2() { return w + kW1 + kHid; }
    float *B2() { return w + kW1 + kHid + kW2; }
    float *W3() { return w + kW1 + kHid + kW2 + kHid; }
    float *B3() { return w + kW1 + kHid + kW2 + kHid + kW3; }
    const __nv_bfloat16 *W1h() const { return wh; }
    const __nv_bfloat16 *W2h() const { return wh + kW1 + kHid; }
    const __nv_bfloat16 *W3h() const { return wh + kW1 + kHid + kW2 + kHid; }
};

#define SCK(call)                                                         \
    do {                                                                  \
        cudaError_t _e = (call);                                          \
        if (_e != cudaSuccess) { set_error(cuda_msg(_e, #call)); return 1; } \
    } while (0)

static cudaError_t refresh_bf16(imfcs_surrogate *h, cudaStream_t s)
{
    to_bf16_kernel<<<(unsigned)((kParams + 255) / 256), 256, 0, s>>>(h->w, h->wh, kParams);
    return cudaGetLastError();
}

// forward over n rows of xh (BF16 [n][128]); y standardised FP32 [n][4]
static cudaError_t forward(imfcs_surrogate *h, int n, cudaStream_t s)
{
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.M = n; g.N = kHid; g.K = kIn;
    g.A = h->xh; g.lam = kIn; g.lak = 1;
    g.B = h->W1h(); g.lbk = kHid; g.lbn = 1;
    g.bias = h->B1(); g.outf = h->z1; g.outh = h->h1;
    cudaError_t e = gemm<EPI_BIAS_GELU>(g, s);
    if (e != cudaSuccess) return e;
    g.K = kHid;
    g.A = h->h1; g.lam = kHid;
    g.B = h->W2h(); g.lbk = kHid;
    g.bias = h->B2(); g.outf = h->z2; g.outh = h->h2;
    if ((e = gemm<EPI_BIAS_GELU>(g, s)) != cudaSuccess) return e;
    g.N = kOut;
    g.A = h->h2;
    g.B = h->W3h(); g.lbk = kOut; g.lbn = 1;
    g.bias = h->B3(); g.outf = h->y; g.outh = nullptr;
    return gemm<EPI_BIAS>(g, s);
}

// backward of the MSE loss against h->tn (standardised targets) into h->grad;
// the mean loss accumulates into *loss (zeroed by the caller)
static cudaError_t backward(imfcs_surrogate *h, int n, double *loss, cudaStream_t s)
{
    cudaError_t e;
    mse_kernel<<<(n * kOut + 255) / 256, 256, 0, s>>>(h->y, h->tn, n, h->dy, h->dyh, loss);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    float *gW1 = h->grad, *gB1 = gW1 + kW1, *gW2 = gB1 + kHid, *gB2 = gW2 + kW2, *gW3 = gB2 + kHid,
          *gB3 = gW3 + kW3;
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.alpha = 1.f;
    // dW3 = h2^T dy  [256 x 4], K = n
    g.M = kHid; g.N = kOut; g.K = n;
    g.A = h->h2; g.lam = 1; g.lak = kHid;
    g.B = h->dyh; g.lbk = kOut; g.lbn = 1;
    g.outf = gW3;
    if ((e = gemm<EPI_STORE>(g, s)) != cudaSuccess) return e;
    colsum_kernel<float><<<kOut, 256, 0, s>>>(h->dy, n, kOut, gB3);
    // dz2 = (dy W3^T) * GELU'(z2)  [n x 256], K = 4
    g.M = n; g.N = kHid; g.K = kOut;
    g.A = h->dyh; g.lam = kOut; g.lak = 1;
    g.B = h->W3h(); g.lbk = 1; g.lbn = kOut;
    g.zin = h->z2; g.outh = h->dz2;
    if ((e = gemm<EPI_GELU_BWD>(g, s)) != cudaSuccess) return e;
    // dW2 = h1^T dz2 [256 x 256], K = n
    g.M = kHid; g.N = kHid; g.K = n;
    g.A = h->h1; g.lam = 1; g.lak = kHid;
    g.B = h->dz2; g.lbk = kHid; g.lbn = 1;
    g.outf = gW2;
    if ((e = gemm<EPI_STORE>(g, s)) != cudaSuccess) return e;
    colsum_kernel<__nv_bfloat16><<<kHid, 256, 0, s>>>(h->dz2, n, kHid, gB2);
    // dz1 = (dz2 W2^T) * GELU'(z1) [n x 256], K = 256
    g.M = n; g.N = kHid; g.K = kHid;
    g.A = h->dz2; g.lam = kHid; g.lak = 1;
    g.B = h->W2h(); g.lbk = 1; g.lbn = kHid;
    g.zin = h->z1; g.outh = h->dz1;
    if ((e = gemm<EPI_GELU_BWD>(g, s)) != cudaSuccess) return e;
    // dW1 = x^T dz1 [128 x 256], K = n
    g.M = kIn; g.N = kHid; g.K = n;
    g.A = h->xh; g.lam = 1; g.lak = kIn;
    g.B = h->dz1; g.lbk = kHid; g.lbn = 1;
    g.outf = gW1;
    if ((e = gemm<EPI_STORE>(g, s)) != cudaSuccess) return e;
    colsum_kernel<__nv_bfloat16><<<kHid, 256, 0, s>>>(h->dz1, n, kHid, gB1);
    return cudaGetLastError();
}

// standardise targets t [n][4] into h->tn
__global__ void standardise_kernel(const float *t, int n, float m0, float m1, float m2, float m3, float s0, float s1,
                                   float s2, float s3, float *tn)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kOut) return;
    const int c = i % kOut;
    const float m = c == 0 ? m0 : c == 1 ? m1 : c == 2 ? m2 : m3, sd = c == 0 ? s0 : c == 1 ? s1 : c == 2 ? s2 : s3;
    tn[i] = (t[i] - m) / sd;
}

__global__ void destandardise_kernel(const float *y, int n, float m0, float m1, float m2, float m3, float s0,
                                     float s1, float s2, float s3, float *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kOut) return;
    const int c = i % kOut;
    const float m = c == 0 ? m0 : c == 1 ? m1 : c == 2 ? m2 : m3, sd = c == 0 ? s0 : c == 1 ? s1 : c == 2 ? s2 : s3;
    out[i] = y[i] * sd + m;
}

static cudaError_t load_batch(imfcs_surrogate *h, const float *x, const float *t, int n, cudaStream_t s)
{
    to_bf16_kernel<<<(unsigned)(((size_t)n * kIn + 255) / 256), 256, 0, s>>>(x, h->xh, (size_t)n * kIn);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !t) return e;
    standardise_kernel<<<(n * kOut + 255) / 256, 256, 0, s>>>(t, n, h->tmean[0], h->tmean[1], h->tmean[2], h->tmean[3],
                                                              h->tstd[0], h->tstd[1], h->tstd[2], h->tstd[3], h->tn);
    return cudaGetLastError();
}

extern "C" size_t imfcs_surrogate_param_count(void) { return kParams; }

extern "C" int imfcs_surrogate_create(uint64_t seed, imfcs_surrogate **out)
{
    if (!out) { set_error("null handle pointer"); return 1; }
    *out = nullptr;
    imfcs_surrogate *h = new imfcs_surrogate();
    cudaError_t e = h->alloc(h->w, kParams);
    if (e == cudaSuccess) e = h->alloc(h->grad, kParams);
    if (e == cudaSuccess) e = h->alloc(h->m, kParams);
    if (e == cudaSuccess) e = h->alloc(h->v, kParams);
    if (e == cudaSuccess) e = h->alloc(h->wh, kParams);
    if (e == cudaSuccess) e = h->alloc(h->loss, 1);
    if (e != cudaSuccess) {
        set_error(cuda_msg(e, "surrogate allocation"));
        delete h;
        return 1;
    }
    // He-style initialisation (seeded), zero biases
    std::vector<float> w(kParams, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](size_t off, size_t n, int fan_in) {
        std::normal_distribution<float> nd(0.f, sqrtf(2.f / (float)fan_in));
        for (size_t i = 0; i < n; i++) w[off + i] = nd(rng);
    };
    fill(0, kW1, kIn);
    fill(kW1 + kHid, kW2, kHid);
    fill(kW1 + kHid + kW2 + kHid, kW3, kHid);
    e = cudaMemcpy(h->w, w.data(), kParams * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->m, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(h->v, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = refresh_bf16(h, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        set_error(cuda_msg(e, "surrogate initialisation"));
        delete h;
        return 1;
    }
    *out = h;
    return 0;
}

extern "C" int imfcs_surrogate_destroy(imfcs_surrogate *h)
{
    delete h;
    return 0;
}

// host_params: kParams FP32 (W1 b1 W2 b2 W3 b3) + 8 (target means, stds)
extern "C" int imfcs_surrogate_get_params(const imfcs_surrogate *h, float *host_params)
{
    if (!h || !host_params) { set_error("null argument"); return 1; }
    SCK(cudaMemcpy(host_params, h->w, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    for (int c = 0; c < kOut; c++) { host_params[kParams + c] = h->tmean[c]; host_params[kParams + kOut + c] = h->tstd[c]; }
    return 0;
}

extern "C" int imfcs_surrogate_set_params(imfcs_surrogate *h, const float *host_params)
{
    if (!h || !host_params) { set_error("null argument"); return 1; }
    SCK(cudaMemcpy(h->w, host_params, kParams * sizeof(float), cudaMemcpyHostToDevice));
    for (int c = 0; c < kOut; c++) { h->tmean[c] = host_params[kParams + c]; h->tstd[c] = host_params[kParams + kOut + c]; }
    SCK(refresh_bf16(h, 0));
    SCK(cudaDeviceSynchronize());
    return 0;
}

extern "C" int imfcs_surrogate_features(int npix, int chanum, const double *dev_acf, const double *dev_var,
                                        float *dev_x, void *stream)
{
    if (npix <= 0 || chanum < kLagsIn + 1 || !dev_acf || !dev_var || !dev_x) {
        set_error("imfcs_surrogate_features: needs at least 65 correlation channels (lags 1..64)");
        return 1;
    }
    features_kernel<<<npix, kLagsIn, 0, (cudaStream_t)stream>>>(npix, chanum, dev_acf, dev_var, dev_x);
    SCK(cudaGetLastError());
    return 0;
}

// One forward + backward pass over n samples; gradients (FP32, kParams) to
// host_grads and the mean loss to *loss.  Uses the current target
// standardisation.
extern "C" int imfcs_surrogate_gradients(imfcs_surrogate *h, const float *dev_x, const float *dev_t, int n,
                                         float *host_grads, double *loss)
{
    if (!h || !dev_x || !dev_t || n <= 0) { set_error("invalid argument"); return 1; }
    SCK(h->reserve(n));
    SCK(load_batch(h, dev_x, dev_t, n, 0));
    SCK(cudaMemset(h->loss, 0, sizeof(double)));
    SCK(forward(h, n, 0));
    SCK(backward(h, n, h->loss, 0));
    if (host_grads) SCK(cudaMemcpy(host_grads, h->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) SCK(cudaMemcpy(loss, h->loss, sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

// Adam training on n samples (dev_x [n][128], dev_t [n][4] raw targets):
// the target standardisation is set from the data, then `steps` minibatch
// steps of `batch` consecutive samples starting at a seeded random offset.
// loss_history (optional, [steps]) receives the minibatch losses.
extern "C" int imfcs_surrogate_train(imfcs_surrogate *h, const float *dev_x, const float *dev_t, int n, int steps,
                                     int batch, float lr, uint64_t seed, float *loss_history, void *stream)
{
    if (!h || !dev_x || !dev_t || n <= 0 || steps <= 0 || batch <= 0) { set_error("invalid argument"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    if (batch > n) batch = n;
    SCK(h->reserve(batch));
    // target standardisation from the data (host side, one pass)
    {
        std::vector<float> t((size_t)n * kOut);
        SCK(cudaMemcpy(t.data(), dev_t, t.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (int c = 0; c < kOut; c++) {
            double s1 = 0, s2 = 0;
            for (int i = 0; i < n; i++) { const double v = t[(size_t)i * kOut + c]; s1 += v; s2 += v * v; }
            const double mean = s1 / n, var = s2 / n - mean * mean;
            h->tmean[c] = (float)mean;
            h->tstd[c] = var > 1e-12 ? (float)sqrt(var) : 1.f;
        }
    }
    std::mt19937_64 rng(seed);
    double *dloss = nullptr;   // per-step minibatch losses, read once at the end
    SCK(cudaMallocAsync((void **)&dloss, sizeof(double) * steps, s));
    cudaError_t e = cudaMemsetAsync(dloss, 0, sizeof(double) * steps, s);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < steps && e == cudaSuccess; it++) {
        const int off = n > batch ? (int)(rng() % (uint64_t)(n - batch + 1)) : 0;
        e = load_batch(h, dev_x + (size_t)off * kIn, dev_t + (size_t)off * kOut, batch, s);
        if (e == cudaSuccess) e = forward(h, batch, s);
        if (e == cudaSuccess) e = backward(h, batch, dloss + it, s);
        if (e != cudaSuccess) break;
        h->adam_t++;
        const float c1 = 1.f / (1.f - powf(b1, (float)h->adam_t)), c2 = 1.f / (1.f - powf(b2, (float)h->adam_t));
        adam_kernel<<<(unsigned)((kParams + 255) / 256), 256, 0, s>>>(h->w, h->grad, h->m, h->v, kParams, lr, b1, b2,
                                                                       eps, c1, c2);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = refresh_bf16(h, s);
    }
    std::vector<double> lh(steps, 0.0);
    if (e == cudaSuccess && loss_history)
        e = cudaMemcpyAsync(lh.data(), dloss, sizeof(double) * steps, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(dloss, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "imfcs_surrogate_train")); return 1; }
    if (loss_history)
        for (int it = 0; it < steps; it++) loss_history[it] = (float)lh[it];
    return 0;
}

// Predictions (de-standardised) for n samples: dev_out [n][4] = log D,
// log(N G1), G_inf / G1, fraction.
extern "C" int imfcs_surrogate_predict(imfcs_surrogate *h, const float *dev_x, int n, float *dev_out, void *stream)
{
    if (!h || !dev_x || !dev_out || n <= 0) { set_error("invalid argument"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    SCK(h->reserve(n));
    SCK(load_batch(h, dev_x, nullptr, n, s));
    SCK(forward(h, n, s));
    destandardise_kernel<<<(n * kOut + 255) / 256, 256, 0, s>>>(h->y, n, h->tmean[0], h->tmean[1], h->tmean[2],
                                                                h->tmean[3], h->tstd[0], h->tstd[1], h->tstd[2],
                                                                h->tstd[3], dev_out);
    SCK(cudaGetLastError());
    return 0;
}

namespace imfcs {
// plan glue (imfcs_capi.cu): features + prediction + per-pixel LM seeds
int surrogate_reserve(imfcs_surrogate *h, int n)
{
    const cudaError_t e = h->reserve(n);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "surrogate work buffers")); return 1; }
    return 0;
}

int surrogate_seed(imfcs_surrogate *h, int npix, int chanum, int k, const int *idx, const double *acf,
                   const double *var, float *x, float *pred, const float *base_init, float *init, cudaStream_t s)
{
    if (imfcs_surrogate_features(npix, chanum, acf, var, x, s)) return 1;
    if (imfcs_surrogate_predict(h, x, npix, pred, s)) return 1;
    FreeIdx f;
    f.k = k;
    for (int i = 0; i < IMFCS_NPARAM; i++) f.idx[i] = i < k ? idx[i] : 0;
    seed_kernel<<<(npix + 127) / 128, 128, 0, s>>>(npix, chanum, f, acf, pred, base_init, init);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(cuda_msg(e, "seed_kernel")); return 1; }
    return 0;
}
}  // namespace imfcs
