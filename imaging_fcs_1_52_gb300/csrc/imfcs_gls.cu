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
// and L^-1.
//
// One pass over the centred samples e_xz gives, per lag pair (x >= y),
// S1 = sum_z e_x e_y and S2 = sum_z (e_x e_y)^2 (FP32 per chunk of samples,
// float-float across chunks; each thread owns a 4x4 tile of pairs, so a
// sample loaded from shared memory serves four pairs).  The shrinkage sums follow
// without a second pass:
//   sum_z (e_x^2 - c_xx)^2               = S2_xx - (pnum - 2) c_xx^2
//   sum_z (e_x e_y / (sd_x sd_y) - r_xy)^2 = (S2_xy - (pnum - 2) c_xy^2) / (c_xx c_yy)
// with c = S1 / (pnum - 1) and r = c / (sd_x sd_y).  Divisions by per-lag
// quantities are multiplications by their reciprocals; the median is a
// parallel rank selection; the FP64 Cholesky's updates spread over the whole
// CTA on the packed lower triangle in shared memory.  GB300 issues FP64 at
// 1/64 of the FP32 rate, so what needs more than FP32 but not the
// FP64 Cholesky -- the centred samples, the sums across chunks,
// L^-1 (one column per thread) and L^-1 mcov -- runs in float-float
// (compensated products and sums, about 44 bits) on the FP32 pipe; L^-1
// leaves the kernel as FP32.
#include <math.h>

#include "imfcs_internal.cuh"
#include "imfcs_args.h"
#include "imfcs_ff.cuh"

namespace imfcs {

constexpr int kGlsThreads = 256;
constexpr int kGlsZChunk = 80;                  // samples per staged chunk
constexpr int kGlsZStride = kGlsZChunk + 1;     // odd row stride: rows in distinct banks
constexpr int kMaxN1 = 96;                      // chanum - 1 limit of this kernel
constexpr int kGlsTile = 4;                     // pairs per thread: 4 x 4

__device__ __forceinline__ int tri(int r, int c) { return r * (r + 1) / 2 + c; }   // c <= r

// Compensated dot-product step (float-float operands a, b; sum (sh, sl)):
// the error of the product and of the running sum go to sl, so the result
// carries about twice the FP32 precision, on the FP32 pipe.  Explicitly
// rounded operations: a contracted sh + ah*bh would break the two-sum.
__device__ __forceinline__ void ff_dot_step(float ah, float al, float bh, float bl, float &sh, float &sl)
{
    const float p = __fmul_rn(ah, bh);
    const float pe = __fadd_rn(fmaf(ah, bh, -p), fmaf(ah, bl, __fmul_rn(al, bh)));
    const float t = __fadd_rn(sh, p);
    const float bb = __fsub_rn(t, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    sl = __fadd_rn(sl, __fadd_rn(e, pe));
    sh = t;
}

__global__ void __launch_bounds__(kGlsThreads) gls_kernel(GlsArgs g)
{
    extern __shared__ double gsh[];
    const int n1 = g.chanum - 1;
    const int npairs = n1 * (n1 + 1) / 2;
    const int nrt = (n1 + kGlsTile - 1) / kGlsTile;    // tile rows
    double *lp = gsh;                  // [npairs] covariance/correlation -> regularised -> Cholesky factor
    double *s2 = gsh + npairs;         // [npairs] S2 -> t_xy
    float2 *a1s = (float2 *)lp, *a2s = (float2 *)s2;   // S1, S2 in float-float during the sample pass
    float *eb = (float *)(gsh + 2 * npairs);   // [nrt*4][kGlsZStride] one chunk of centred samples
    float *lh = eb, *ll = eb + npairs;         // L in float-float (after the Cholesky)
    float *xh = (float *)s2, *xl = xh + npairs;   // L^-1 in float-float
    __shared__ double mcov[kMaxN1], inv_dm[kMaxN1], cdiag[kMaxN1], isd[kMaxN1], sq[kMaxN1], rdiag[kMaxN1];
    __shared__ f2 inv_dmf[kMaxN1], mcovf[kMaxN1], rdf[kMaxN1];
    __shared__ double red[2][kGlsThreads / 32];
    __shared__ double s_med[2], s_lamvar, s_lamcov, s_piv;
    __shared__ int s_fail;

    const int pix = blockIdx.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int pnum = g.pnum_by_ind[g.blk_ind[pix]];
    const float *bp = g.bprod + (size_t)pix * n1 * g.pnum_stride;
    const double inv_pm1 = 1.0 / (double)(pnum - 1), inv_pnum = 1.0 / (double)pnum;
    if (tid < n1) {
        const float4 m = g.mon[(size_t)pix * g.chanum + tid + 1];
        inv_dm[tid] = 1.0 / ((double)m.z * (double)m.w);
        inv_dmf[tid] = f2_from_d(inv_dm[tid]);
    }
    if (tid == 0) s_fail = 0;
    for (int i = tid; i < npairs; i += kGlsThreads) { lp[i] = 0.0; s2[i] = 0.0; }
    // rows past n1 of the staging buffer stay zero
    for (int i = n1 * kGlsZStride + tid; i < nrt * kGlsTile * kGlsZStride; i += kGlsThreads) eb[i] = 0.f;
    // mcov (java:9526-9531): sum of the blocked products (float-float per
    // lane and across the warp), one warp per lag
    for (int x = warp; x < n1; x += kGlsThreads / 32) {
        float sh = 0.f, sl = 0.f;
        for (int z = lane; z < pnum; z += 32) {
            const f2 t = f2_two_sum(sh, bp[(size_t)x * g.pnum_stride + z]);
            sh = t.hi;
            sl = __fadd_rn(sl, t.lo);
        }
        f2 sum = f2_two_sum(sh, sl);
        for (int o = 16; o > 0; o >>= 1) {
            const f2 other = {__shfl_xor_sync(0xffffffffu, sum.hi, o), __shfl_xor_sync(0xffffffffu, sum.lo, o)};
            sum = f2_add(sum, other);
        }
        if (lane == 0) mcov[x] = (double)sum.hi + (double)sum.lo;
    }
    __syncthreads();                  // inv_dm (threads < n1) and the sums (warps)
    if (tid < n1) {
        mcov[tid] = mcov[tid] * inv_dm[tid] * inv_pnum;
        mcovf[tid] = f2_from_d(mcov[tid]);
    }
    __syncthreads();

    // S1, S2 per pair: thread t owns tile (bx, by), bx >= by, of the pairs
    // x in [4 bx, 4 bx + 4), y in [4 by, 4 by + 4)
    const int ntiles = nrt * (nrt + 1) / 2;
    for (int t0 = 0; t0 < ntiles; t0 += kGlsThreads) {
        const int t = t0 + tid;
        int bx = 0, by = 0;
        if (t < ntiles) {
            bx = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
            while ((bx + 1) * (bx + 2) / 2 <= t) bx++;
            while (bx * (bx + 1) / 2 > t) bx--;
            by = t - bx * (bx + 1) / 2;
        }
        for (int z0 = 0; z0 < pnum; z0 += kGlsZChunk) {
            const int zn = min(kGlsZChunk, pnum - z0);
            __syncthreads();
            // centred sample e = b / (dm Dm) - mcov in float-float: the
            // product exactly as hi + lo, then the subtraction of the mean
            for (int i = tid; i < n1 * kGlsZChunk; i += kGlsThreads) {
                const int x = i / kGlsZChunk, z = i - x * kGlsZChunk;
                if (z < zn) {
                    const float b = bp[(size_t)x * g.pnum_stride + z0 + z];
                    const f2 iv = inv_dmf[x], mc = mcovf[x];
                    const float ph = __fmul_rn(b, iv.hi);
                    const float pl = fmaf(b, iv.lo, fmaf(b, iv.hi, -ph));
                    eb[x * kGlsZStride + z] = __fadd_rn(__fsub_rn(ph, mc.hi), __fsub_rn(pl, mc.lo));
                }
            }
            __syncthreads();
            if (t >= ntiles) continue;
            float a1[kGlsTile][kGlsTile], a2[kGlsTile][kGlsTile];
#pragma unroll
            for (int i = 0; i < kGlsTile; i++)
#pragma unroll
                for (int j = 0; j < kGlsTile; j++) { a1[i][j] = 0.f; a2[i][j] = 0.f; }
            const float *ex = eb + (kGlsTile * bx) * kGlsZStride, *ey = eb + (kGlsTile * by) * kGlsZStride;
            for (int z = 0; z < zn; z++) {
                float vx[kGlsTile], vy[kGlsTile];
#pragma unroll
                for (int i = 0; i < kGlsTile; i++) { vx[i] = ex[i * kGlsZStride + z]; vy[i] = ey[i * kGlsZStride + z]; }
#pragma unroll
                for (int i = 0; i < kGlsTile; i++)
#pragma unroll
                    for (int j = 0; j < kGlsTile; j++) {
                        const float u = vx[i] * vy[j];
                        a1[i][j] += u;
                        a2[i][j] = fmaf(u, u, a2[i][j]);
                    }
            }
#pragma unroll
            for (int i = 0; i < kGlsTile; i++)
#pragma unroll
                for (int j = 0; j < kGlsTile; j++) {
                    const int x = kGlsTile * bx + i, y = kGlsTile * by + j;
                    if (x < n1 && y <= x) {
                        float2 v = a1s[tri(x, y)];
                        f2 sv = f2_two_sum(v.x, a1[i][j]);
                        a1s[tri(x, y)] = make_float2(sv.hi, __fadd_rn(v.y, sv.lo));
                        v = a2s[tri(x, y)];
                        sv = f2_two_sum(v.x, a2[i][j]);
                        a2s[tri(x, y)] = make_float2(sv.hi, __fadd_rn(v.y, sv.lo));
                    }
                }
        }
    }
    __syncthreads();
    // covariance (java:9534-9542), S2 in FP64, standard deviations
    for (int i = tid; i < npairs; i += kGlsThreads) {
        const float2 v = a1s[i], w = a2s[i];
        lp[i] = ((double)v.x + (double)v.y) * inv_pm1;
        s2[i] = (double)w.x + (double)w.y;
    }
    __syncthreads();
    if (tid < n1) {
        const double c = lp[tri(tid, tid)];
        cdiag[tid] = c;
        isd[tid] = 1.0 / sqrt(c);
    }
    __syncthreads();
    // median of the chanum diagonal entries incl. the zero-lag slot that
    // stays 0 (java:9563-9573): rank selection, ties ordered by index
    if (tid <= n1) {
        const double v = tid == 0 ? 0.0 : cdiag[tid - 1];
        int rank = 0;
        for (int j = 0; j <= n1; j++) {
            const double w = j == 0 ? 0.0 : cdiag[j - 1];
            rank += (w < v) || (w == v && j < tid);
        }
        const int c = n1 + 1;
        const int pos1 = (c - 1) / 2, pos2 = c / 2;     // floor / ceil of (c - 1) / 2
        if (rank == pos1) s_med[0] = v;
        if (rank == pos2) s_med[1] = v;
    }
    // t_xy and correlations; lamvar's and lamcov's sums
    const double f = (double)pnum / pow((double)pnum - 1.0, 3);
    const double pm2 = (double)(pnum - 2);
    for (int i = tid; i < npairs; i += kGlsThreads) {
        int x = (int)((sqrtf(8.f * i + 1.f) - 1.f) * 0.5f);
        while ((x + 1) * (x + 2) / 2 <= i) x++;
        while (x * (x + 1) / 2 > i) x--;
        const int y = i - x * (x + 1) / 2;
        const double c = lp[i];
        const double t = s2[i] - pm2 * c * c;        // sum_z (e_x e_y - c_xy)^2 terms
        if (x == y) {
            s2[i] = t;                               // lamvar numerator term
        } else {
            const double k = isd[x] * isd[y];
            s2[i] = t * k * k;                       // t_xy
            lp[i] = c * k;                           // correlation
        }
    }
    __syncthreads();
    if (tid == 0) {
        const double med = (s_med[0] + s_med[1]) * 0.5;
        s_med[0] = med;
    }
    {
        double num = 0.0, den = 0.0;
        if (tid < n1) num = s2[tri(tid, tid)] * f;
        __syncthreads();                              // the median's average
        if (tid < n1) {
            const double d = cdiag[tid] - s_med[0];
            den = d * d;
        }
        num = warp_sum_d(num);
        den = warp_sum_d(den);
        if (lane == 0) { red[0][warp] = num; red[1][warp] = den; }
        __syncthreads();
        if (tid == 0) {
            double a = 0.0, b = 0.0;
            for (int w = 0; w < kGlsThreads / 32; w++) { a += red[0][w]; b += red[1][w]; }
            s_lamvar = fmax(fmin(1.0, a / b), 0.0);
        }
        __syncthreads();
    }
    // lamcov: per x, T_y = (T_{y-1} + t_xy) f summed over y < x
    {
        double num = 0.0, den = 0.0;
        if (tid < n1) {
            const int x = tid;
            double T = 0.0;
            for (int y = 0; y < x; y++) {
                T = (T + s2[tri(x, y)]) * f;
                num += T;
                const double r = lp[tri(x, y)];
                den += r * r;
            }
        }
        num = warp_sum_d(num);
        den = warp_sum_d(den);
        if (lane == 0) { red[0][warp] = num; red[1][warp] = den; }
        __syncthreads();
        if (tid == 0) {
            double a = 0.0, b = 0.0;
            for (int w = 0; w < kGlsThreads / 32; w++) { a += red[0][w]; b += red[1][w]; }
            s_lamcov = fmax(fmin(1.0, a / b), 0.0);
        }
        __syncthreads();
    }
    // regularised covariance (java:9605-9615), FP64, packed lower triangle
    const double lv = s_lamvar, lc = s_lamcov, med = s_med[0];
    if (tid < n1) {
        const double d = lv * med + (1.0 - lv) * cdiag[tid];
        sq[tid] = sqrt(d);
        rdiag[tid] = d * inv_pnum;
    }
    __syncthreads();
    for (int i = tid; i < npairs; i += kGlsThreads) {
        int x = (int)((sqrtf(8.f * i + 1.f) - 1.f) * 0.5f);
        while ((x + 1) * (x + 2) / 2 <= i) x++;
        while (x * (x + 1) / 2 > i) x--;
        const int y = i - x * (x + 1) / 2;
        lp[i] = (x == y) ? rdiag[x] : (1.0 - lc) * lp[i] * sq[x] * sq[y] * inv_pnum;
    }
    __syncthreads();
    if (g.covmats_out)
        for (int i = tid; i < n1 * n1; i += kGlsThreads) {
            const int x = i / n1, y = i - x * n1;
            g.covmats_out[(size_t)pix * n1 * n1 + i] = x >= y ? lp[tri(x, y)] : lp[tri(y, x)];
        }
    // Cholesky in commons-math's order (java:13717): pivot i, scale its
    // column, then the trailing update A[q][p] -= A[q][i] A[p][i] (p <= q),
    // FP64.  The pivot's 1/sqrt by Newton-Raphson from an FP32 estimate
    // (two steps: ~1e-16), sqrt(d) = d / sqrt(d) corrected once; the update
    // spreads its (q, p) over the whole CTA.
    for (int i = 0; i < n1; i++) {
        if (tid == 0) {
            const double d = lp[tri(i, i)];
            if (!(d > 1e-10)) {
                s_fail = 1;
            } else {
                double rs, r;
                if (d < 1e30) {
                    rs = (double)rsqrtf((float)d);
                    rs = rs * fma(-0.5 * d * rs, rs, 1.5);
                    rs = rs * fma(-0.5 * d * rs, rs, 1.5);
                    r = d * rs;
                    r = fma(0.5 * rs, fma(-r, r, d), r);
                } else {
                    r = sqrt(d);
                    rs = 1.0 / r;
                }
                lp[tri(i, i)] = r;
                s_piv = rs;
                rdiag[i] = rs;
            }
        }
        __syncthreads();
        if (s_fail) break;
        for (int q = i + 1 + tid; q < n1; q += kGlsThreads) lp[tri(q, i)] *= s_piv;
        __syncthreads();
        const int m = n1 - 1 - i;
        const int cnt = m * (m + 1) / 2;
        for (int e = tid; e < cnt; e += kGlsThreads) {
            int a = (int)((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
            while ((a + 1) * (a + 2) / 2 <= e) a++;
            while (a * (a + 1) / 2 > e) a--;
            const int q = i + 1 + a, pp = i + 1 + (e - a * (a + 1) / 2);
            lp[tri(q, pp)] -= lp[tri(q, i)] * lp[tri(pp, i)];
        }
        __syncthreads();
    }
    if (s_fail) {
        if (tid == 0) g.ok[pix] = 0;
        return;
    }
    // L and 1/diag(L) in float-float for the triangular inverse on the FP32
    // pipe (the output L^-1 is FP32)
    for (int i = tid; i < npairs; i += kGlsThreads) {
        const double v = lp[i];
        const float hi = (float)v;
        lh[i] = hi;
        ll[i] = (float)(v - (double)hi);
    }
    if (tid < n1) rdf[tid] = f2_from_d(rdiag[tid]);
    __syncthreads();
    // L^-1, column c on thread c: X[c][c] = 1/L[c][c],
    // X[r][c] = -(sum_{m=c}^{r-1} L[r][m] X[m][c]) / L[r][r]
    if (tid < n1) {
        const int c = tid;
        xh[tri(c, c)] = rdf[c].hi;
        xl[tri(c, c)] = rdf[c].lo;
        for (int r = c + 1; r < n1; r++) {
            const int rb = tri(r, 0);
            float sh = 0.f, sl = 0.f;
            int xi = tri(c, c);
            for (int m = c; m < r; m++) {
                ff_dot_step(lh[rb + m], ll[rb + m], xh[xi], xl[xi], sh, sl);
                xi += m + 1;
            }
            const f2 x = f2_mul(f2_two_sum(sh, sl), rdf[r]);
            xh[tri(r, c)] = -x.hi;
            xl[tri(r, c)] = -x.lo;
        }
    }
    __syncthreads();
    float *lo = g.linv + (size_t)pix * npairs;
    for (int i = tid; i < npairs; i += kGlsThreads) lo[i] = __fadd_rn(xh[i], xl[i]);
    // transformed data L^-1 mcov
    if (tid < n1) {
        const int r = tid, rb = tri(r, 0);
        float sh = 0.f, sl = 0.f;
        for (int c = 0; c <= r; c++) ff_dot_step(xh[rb + c], xl[rb + c], mcovf[c].hi, mcovf[c].lo, sh, sl);
        g.ytrans[(size_t)pix * n1 + r] = sh + sl;
    }
    if (tid == 0) g.ok[pix] = 1;
}

size_t gls_smem_bytes(int chanum)
{
    const int n1 = chanum - 1;
    const size_t npairs = (size_t)n1 * (n1 + 1) / 2;
    const size_t rows = (size_t)((n1 + kGlsTile - 1) / kGlsTile) * kGlsTile;
    const size_t stage = rows * kGlsZStride * sizeof(float);
    return 2 * npairs * sizeof(double) + (stage > npairs * sizeof(double) ? stage : npairs * sizeof(double));
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
