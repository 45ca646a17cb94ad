// imfcs_gls.cu -- regularised covariance of the ACF and its Cholesky factor
// for the GLS fit.  One CTA per pixel.
//
// Restates the GLS branch of calculateCF (Imaging_FCS_1_52.java:9524-9610):
// the blocked products of lags 1..C-1 (first pnum blocks, from the
// correlator) normalised by dm*Dm, their mean mcov, the sample covariance,
// the shrinkage weights lamvar (variance towards the median, which includes
// the unset zero-lag slot, java:9563-9573) and lamcov (correlations towards
// zero, with the Java accumulation order, java:9592-9603), then the FP64
// Cholesky with commons-math's thresholds (dataTransform, java:13705-13729)
// and L^-1.  Products and first sums are FP32 with FP64 chunk accumulation;
// the regularisation, Cholesky and inverse are FP64.
#include <math.h>

#include "imfcs_internal.cuh"
#include "imfcs_args.h"

namespace imfcs {

constexpr int kGlsThreads = 256;
constexpr int kGlsZChunk = 128;
constexpr int kMaxN1 = 96;   // chanum - 1 limit of this kernel



__device__ __forceinline__ void pair_of(int pr, int &x, int &y)
{
    int xx = (int)((sqrtf(8.f * pr + 1.f) - 1.f) * 0.5f);
    while ((xx + 1) * (xx + 2) / 2 <= pr) xx++;
    while (xx * (xx + 1) / 2 > pr) xx--;
    x = xx;
    y = pr - xx * (xx + 1) / 2;
}

__global__ void __launch_bounds__(kGlsThreads) gls_kernel(GlsArgs g)
{
    extern __shared__ double gsh[];
    const int n1 = g.chanum - 1;
    const int npairs = n1 * (n1 + 1) / 2;
    double *cm = gsh;                                  // [n1][n1] covmats / t_xy scratch
    float *zb = (float *)(gsh + n1 * n1);              // [n1][kGlsZChunk]
    __shared__ double mcov[kMaxN1], dmdm[kMaxN1], cdiag[kMaxN1], sdiag[kMaxN1];
    __shared__ double red[kGlsThreads / 32];
    __shared__ double s_median, s_lamvar, s_lamcov;
    __shared__ int s_fail;

    const int pix = blockIdx.x;
    const int tid = threadIdx.x;
    const int pnum = g.pnum_by_ind[g.blk_ind[pix]];
    const float *bp = g.bprod + (size_t)pix * n1 * g.pnum_stride;
    if (tid < n1) {
        float4 m = g.mon[(size_t)pix * g.chanum + tid + 1];
        dmdm[tid] = (double)m.z * (double)m.w;
    }
    if (tid == 0) s_fail = 0;
    __syncthreads();
    // mcov (java:9526-9531)
    if (tid < n1) {
        double s = 0.0;
        for (int z = 0; z < pnum; z++) s += (double)bp[(size_t)tid * g.pnum_stride + z] / dmdm[tid];
        mcov[tid] = s / pnum;
    }
    __syncthreads();
    // covariance (java:9534-9542): pairs (x >= y)
    constexpr int kMaxPairsPerThread = (kMaxN1 * (kMaxN1 + 1) / 2 + kGlsThreads - 1) / kGlsThreads;
    double cacc[kMaxPairsPerThread];
    for (int r = 0; r < kMaxPairsPerThread; r++) cacc[r] = 0.0;
    for (int z0 = 0; z0 < pnum; z0 += kGlsZChunk) {
        int zn = min(kGlsZChunk, pnum - z0);
        for (int i = tid; i < n1 * kGlsZChunk; i += kGlsThreads) {
            int x = i / kGlsZChunk, z = i % kGlsZChunk;
            zb[i] = z < zn ? (float)((double)bp[(size_t)x * g.pnum_stride + z0 + z] / dmdm[x] - mcov[x]) : 0.f;
        }
        __syncthreads();
        for (int r = 0; r < kMaxPairsPerThread; r++) {
            int pr = tid + r * kGlsThreads;
            if (pr >= npairs) break;
            int x, y;
            pair_of(pr, x, y);
            const float *ex = zb + x * kGlsZChunk, *ey = zb + y * kGlsZChunk;
            float s = 0.f;
            for (int z = 0; z < zn; z++) s = fmaf(ex[z], ey[z], s);
            cacc[r] += (double)s;
        }
        __syncthreads();
    }
    // covariance to cm (full symmetric)
    for (int r = 0; r < kMaxPairsPerThread; r++) {
        int pr = tid + r * kGlsThreads;
        if (pr >= npairs) break;
        int x, y;
        pair_of(pr, x, y);
        double v = cacc[r] / (pnum - 1);
        cm[x * n1 + y] = v;
        cm[y * n1 + x] = v;
    }
    __syncthreads();
    if (tid < n1) { cdiag[tid] = cm[tid * n1 + tid]; sdiag[tid] = sqrt(cdiag[tid]); }
    __syncthreads();
    // median over chanum entries incl. the zero-lag slot that stays 0 (java:9563-9573)
    if (tid == 0) {
        double v[kMaxN1 + 1];
        v[0] = 0.0;
        for (int i = 0; i < n1; i++) v[i + 1] = cdiag[i];
        for (int i = 1; i <= n1; i++) {
            double t = v[i];
            int jj = i - 1;
            while (jj >= 0 && v[jj] > t) { v[jj + 1] = v[jj]; jj--; }
            v[jj + 1] = t;
        }
        int c = n1 + 1;
        double pos1 = floor((c - 1.0) / 2.0), pos2 = ceil((c - 1.0) / 2.0);
        s_median = (pos1 == pos2) ? v[(int)pos1] : (v[(int)pos1] + v[(int)pos2]) / 2.0;
    }
    __syncthreads();
    const double f = (double)pnum / pow((double)pnum - 1.0, 3);
    // shrinkage sums: per-x variance-of-variance, per-pair variance-of-correlation
    double varnum[(kMaxN1 + kGlsThreads - 1) / kGlsThreads] = {0.0};
    double tacc[kMaxPairsPerThread];
    for (int r = 0; r < kMaxPairsPerThread; r++) tacc[r] = 0.0;
    for (int z0 = 0; z0 < pnum; z0 += kGlsZChunk) {
        int zn = min(kGlsZChunk, pnum - z0);
        for (int i = tid; i < n1 * kGlsZChunk; i += kGlsThreads) {
            int x = i / kGlsZChunk, z = i % kGlsZChunk;
            zb[i] = z < zn ? (float)((double)bp[(size_t)x * g.pnum_stride + z0 + z] / dmdm[x] - mcov[x]) : 0.f;
        }
        __syncthreads();
        if (tid < n1) {
            float cxx = (float)cdiag[tid], s = 0.f;
            for (int z = 0; z < zn; z++) { float e = zb[tid * kGlsZChunk + z]; float d = e * e - cxx; s = fmaf(d, d, s); }
            varnum[0] += (double)s;
        }
        for (int r = 0; r < kMaxPairsPerThread; r++) {
            int pr = tid + r * kGlsThreads;
            if (pr >= npairs) break;
            int x, y;
            pair_of(pr, x, y);
            if (y == x) continue;
            const float *ex = zb + x * kGlsZChunk, *ey = zb + y * kGlsZChunk;
            float isx = (float)(1.0 / sdiag[x]), isy = (float)(1.0 / sdiag[y]);
            float cor = (float)(cm[x * n1 + y] / (sdiag[x] * sdiag[y]));
            float s = 0.f;
            for (int z = 0; z < zn; z++) { float d = ex[z] * isx * (ey[z] * isy) - cor; s = fmaf(d, d, s); }
            tacc[r] += (double)s;
        }
        __syncthreads();
    }
    // lamvar
    {
        double num = (tid < n1) ? varnum[0] * f : 0.0;
        double den = (tid < n1) ? (cdiag[tid] - s_median) * (cdiag[tid] - s_median) : 0.0;
        num = warp_sum_d(num);
        den = warp_sum_d(den);
        if ((tid & 31) == 0) red[tid >> 5] = num;
        __syncthreads();
        if (tid == 0) { double s = 0; for (int i = 0; i < kGlsThreads / 32; i++) s += red[i]; s_lamvar = s; }
        __syncthreads();
        if ((tid & 31) == 0) red[tid >> 5] = den;
        __syncthreads();
        if (tid == 0) {
            double s = 0; for (int i = 0; i < kGlsThreads / 32; i++) s += red[i];
            double lv = fmin(1.0, s_lamvar / s);
            s_lamvar = fmax(lv, 0.0);
        }
        __syncthreads();
    }
    // lamcov: t_xy into cm's strictly upper triangle scratch (cm[y*n1+x], y<x), then
    // the Java recursion T_y = (T_{y-1} + t_xy) f, numerator += T_y per x.
    __syncthreads();
    // keep covariance values needed later: store correlations first
    for (int r = 0; r < kMaxPairsPerThread; r++) {
        int pr = tid + r * kGlsThreads;
        if (pr >= npairs) break;
        int x, y;
        pair_of(pr, x, y);
        if (y == x) continue;
        cm[y * n1 + x] = tacc[r];                    // upper: t_xy
        cm[x * n1 + y] = cm[x * n1 + y] / (sdiag[x] * sdiag[y]);   // lower: cor_xy
    }
    __syncthreads();
    {
        double num = 0.0, den = 0.0;
        if (tid < n1) {
            int x = tid;
            double T = 0.0;
            for (int y = 0; y < x; y++) {
                T = (T + cm[y * n1 + x]) * f;
                num += T;
                double c = cm[x * n1 + y];
                den += c * c;
            }
        }
        num = warp_sum_d(num);
        den = warp_sum_d(den);
        __syncthreads();
        if ((tid & 31) == 0) red[tid >> 5] = num;
        __syncthreads();
        double tot_num = 0.0;
        if (tid == 0) for (int i = 0; i < kGlsThreads / 32; i++) tot_num += red[i];
        __syncthreads();
        if ((tid & 31) == 0) red[tid >> 5] = den;
        __syncthreads();
        if (tid == 0) {
            double s = 0; for (int i = 0; i < kGlsThreads / 32; i++) s += red[i];
            double lc = fmin(1.0, tot_num / s);
            s_lamcov = fmax(lc, 0.0);
        }
        __syncthreads();
    }
    // regularised covmats (java:9605-9615), FP64, full matrix in cm
    const double lv = s_lamvar, lc = s_lamcov, med = s_median;
    constexpr int kPer = (kMaxN1 * kMaxN1 + kGlsThreads - 1) / kGlsThreads;
    double vals[kPer];
#pragma unroll
    for (int r = 0; r < kPer; r++) {
        int i = tid + r * kGlsThreads;
        vals[r] = 0.0;
        if (i >= n1 * n1) continue;
        int x = i / n1, y = i % n1;
        if (x == y) continue;
        int xl = x > y ? x : y, yl = x > y ? y : x;
        double cor = cm[xl * n1 + yl];
        double cmx = lv * med + (1 - lv) * cdiag[xl];
        double cmy = lv * med + (1 - lv) * cdiag[yl];
        vals[r] = (1 - lc) * cor * sqrt(cmx * cmy) / pnum;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kPer; r++) {
        int i = tid + r * kGlsThreads;
        if (i < n1 * n1 && (i / n1) != (i % n1)) cm[i] = vals[r];
    }
    __syncthreads();
    if (tid < n1) cm[tid * n1 + tid] = (lv * med + (1 - lv) * cdiag[tid]) / pnum;
    __syncthreads();
    if (g.covmats_out)
        for (int i = tid; i < n1 * n1; i += kGlsThreads) g.covmats_out[(size_t)pix * n1 * n1 + i] = cm[i];
    __syncthreads();
    // Cholesky, commons-math order (java:13717): row-oriented on lt = cm (upper used)
    for (int i = 0; i < n1; i++) {
        if (tid == 0) {
            double d = cm[i * n1 + i];
            if (!(d > 1e-10)) s_fail = 1;
            cm[i * n1 + i] = sqrt(d);
        }
        __syncthreads();
        if (s_fail) break;
        double inv = 1.0 / cm[i * n1 + i];
        for (int q = i + 1 + tid; q < n1; q += kGlsThreads) cm[i * n1 + q] *= inv;
        __syncthreads();
        int m = n1 - i - 1;
        for (int t = tid; t < m * m; t += kGlsThreads) {
            int q = i + 1 + t / m, p = i + 1 + t % m;
            if (p >= q) cm[q * n1 + p] -= cm[i * n1 + q] * cm[i * n1 + p];
        }
        __syncthreads();
    }
    if (s_fail) {
        if (tid == 0) g.ok[pix] = 0;
        return;
    }
    // L = lt^T: L[r][c] = cm[c*n1 + r] for c <= r.  L^-1 column by column.
    float *lo = g.linv + (size_t)pix * npairs;
    if (tid < n1) {
        const int col = tid;
        double xv[kMaxN1];
        for (int r = 0; r < col; r++) xv[r] = 0.0;
        xv[col] = 1.0 / cm[col * n1 + col];
        for (int r = col + 1; r < n1; r++) {
            double s = 0.0;
            for (int m = col; m < r; m++) s += cm[m * n1 + r] * xv[m];
            xv[r] = -s / cm[r * n1 + r];
        }
        for (int r = col; r < n1; r++) lo[(size_t)r * (r + 1) / 2 + col] = (float)xv[r];
    }
    // transformed data L^-1 mcov (forward substitution, FP64)
    if (tid == 0) {
        double yv[kMaxN1];
        for (int r = 0; r < n1; r++) {
            double s = mcov[r];
            for (int m = 0; m < r; m++) s -= cm[m * n1 + r] * yv[m];
            yv[r] = s / cm[r * n1 + r];
            g.ytrans[(size_t)pix * n1 + r] = (float)yv[r];
        }
        g.ok[pix] = 1;
    }
}

size_t gls_smem_bytes(int chanum)
{
    int n1 = chanum - 1;
    return (size_t)n1 * n1 * sizeof(double) + (size_t)n1 * kGlsZChunk * sizeof(float);
}

cudaError_t launch_gls(const GlsArgs &g, cudaStream_t stream)
{
    if (g.chanum - 1 > kMaxN1) return cudaErrorInvalidValue;
    size_t smem = gls_smem_bytes(g.chanum);
    cudaFuncSetAttribute(gls_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    gls_kernel<<<g.npix, kGlsThreads, smem, stream>>>(g);
    return cudaGetLastError();
}

}  // namespace imfcs
