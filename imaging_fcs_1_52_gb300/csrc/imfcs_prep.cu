// imfcs_prep.cu -- the passes in front of the correlator:
//   trace_kernel       averaged intensity trace (calcIntensityTrace, java:9822-9855)
//   bleach_*_kernel    polynomial / exponential bleach fits (java:10845-11004)
//   monitor_finalize_kernel  the lags' monitors from the partial sums the
//                      streaming pass (imfcs_stream.cu) wrote (java:9484-9491)
//   block_kernel       lag-1 blocking curve of blockTransform (java:9217-9422),
//                      from the corrected level-0 stream
// The streaming passes split the time axis into segments so that every SM
// has enough loads in flight.
#include <math.h>

#include "imfcs_internal.cuh"
#include "imfcs_ff.cuh"
#include "imfcs_host.h"

namespace imfcs {

// ---------------------------------------------------------------------------
// Averaged trace: out[trace][x] = (int) sum_{ave frames, window} / ave.
// Block (32 traces) x (8 rows); each thread computes 4 points; a shared tile
// transposes the result so both reads and writes are coalesced.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) trace_kernel(Job j, const void *stack, float *trace_out)
{
    __shared__ float tile[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int trace = blockIdx.x * 32 + tx;
    const int xbase = blockIdx.y * 32;
    int x0 = 0, y0 = 0;
    const bool valid = trace < j.ntrace;
    if (valid) trace_origin(j, trace, x0, y0);
    const int bg = valid ? trace_bg_avg(j, trace) : 0;
    for (int r = 0; r < 4; r++) {
        int xl = ty * 4 + r, x = xbase + xl;
        float val = 0.f;
        if (valid && x < j.nopit) {
            int sum = 0;
            const int fb = x * j.ave, fe = (x + 1) * j.ave;
            for (int f = fb; f < fe; f += 8) {
                float v[8];
                window_values<8>(j, stack, x0, y0, f, fe, bg, v);
#pragma unroll
                for (int u = 0; u < 8; u++) sum += (int)v[u];
            }
            val = (float)(sum / j.ave);
        }
        tile[tx][xl] = val;
    }
    __syncthreads();
    for (int r = 0; r < 4; r++) {
        int tl = ty * 4 + r, tr = blockIdx.x * 32 + tl, x = xbase + tx;
        if (tr < j.ntrace && x < j.nopit) trace_out[(size_t)tr * j.nopit + x] = tile[tl][tx];
    }
}

// ---------------------------------------------------------------------------
// Polynomial bleach fit: least squares in the Legendre basis of
// u = t * uscale + uoff (t = averaged-trace time), coefficients = proj * y
// with the FP64 projection matrix proj[(order+1)][nopit] built on the host.
// One warp per trace.  Also writes f0 = f(0), the centre c and flags.
// ---------------------------------------------------------------------------
__global__ void bleach_poly_kernel(Job j, const float *trace, const double *proj, float uscale,
                                   float uoff, float *bp_out)
{
    const int lane = threadIdx.x & 31;
    const int tr = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (tr >= j.ntrace) return;
    const int k = j.poly_order + 1;
    const float *y = trace + (size_t)tr * j.nopit;
    double c[kMaxPoly + 1];
    for (int i = 0; i < k; i++) c[i] = 0.0;
    for (int x = lane; x < j.nopit; x += 32) {
        double yx = (double)__ldg(&y[x]);
        for (int i = 0; i < k; i++) c[i] = fma(__ldg(&proj[(size_t)i * j.nopit + x]), yx, c[i]);
    }
    for (int i = 0; i < k; i++) c[i] = warp_sum_d(c[i]);
    float cf[kMaxPoly + 1], lb[kMaxPoly + 1];
    for (int i = 0; i < k; i++) cf[i] = (float)c[i];
    legendre(uoff, j.poly_order, lb);    // u(0) = uoff
    double f0 = 0.0;
    for (int i = 0; i < k; i++) f0 += c[i] * (double)lb[i];
    float f0f = (float)f0, inv_f0 = (float)(1.0 / f0);
    // centre: mean of the finite points of the corrected averaged trace (a
    // shift the correlator removes exactly; non-finite points, where the
    // curve crosses zero, are left out so that they cannot spread)
    float csum = 0.f, cnt = 0.f;
    for (int x = lane; x < j.nopit; x += 32) {
        float t = j.frametime * ((float)x + 0.5f) * (float)j.ave;
        legendre(t * uscale + uoff, j.poly_order, lb);
        float f = 0.f;
        for (int i = 0; i < k; i++) f = fmaf(cf[i], lb[i], f);
        const float v = bleach_correct(__ldg(&y[x]), f, f0f, inv_f0);
        if (isfinite(v)) { csum += v; cnt += 1.f; }
    }
    csum = warp_sum(csum);
    cnt = warp_sum(cnt);
    if (lane == 0) {
        float *bp = bp_out + (size_t)tr * kBleachStride;
        for (int i = 0; i < k; i++) bp[i] = cf[i];
        bp[9] = f0f;
        bp[10] = inv_f0;
        bp[11] = (isfinite(f0) && f0 != 0.0) ? 1.f : 0.f;
        bp[12] = cnt > 0.f ? csum / cnt : 0.f;
        bp[13] = uscale;
        bp[14] = uoff;
    }
}

// Centre only (no bleach correction): mean of the averaged trace.
__global__ void center_kernel(Job j, const float *trace, float *bp_out)
{
    const int lane = threadIdx.x & 31;
    const int tr = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (tr >= j.ntrace) return;
    const float *y = trace + (size_t)tr * j.nopit;
    float s = 0.f;
    for (int x = lane; x < j.nopit; x += 32) s += __ldg(&y[x]);
    s = warp_sum(s);
    if (lane == 0) {
        float *bp = bp_out + (size_t)tr * kBleachStride;
        bp[11] = 0.f;
        bp[12] = s / j.nopit;
    }
}

// ---------------------------------------------------------------------------
// Exponential bleach fits (SingleExp / DoubleExp, java:13028-13085).
//
// The reference fits A e^{-t/tau} + C (+ A2 e^{-t/tau2}) by Levenberg-
// Marquardt from fixed initial guesses (java:10862-10864, 10917-10921).  The
// same least-squares problem is solved here in the equivalent parameters
//     f0 = f(0),  s_c = A_c / tau_c,  k_c = 1 / tau_c >= 0,
//     f(t) = f0 - sum_c s_c (1 - e^{-k_c t}) / k_c,
// which stay well conditioned when a component is slow (k_c t << 1, where
// the reference's A and C grow without bound while A + C stays finite) and
// are continuous through k_c = 0 (tau = infinity): the fit is the
// least-squares minimum over k_c >= 0 (a rate at its bound whose step points
// below it is held there), whose linear limit stands for the reference's
// A, tau, C stopping in the tau -> infinity valley.
// Scaled variables t / tmax, y / ymax; one warp per trace.
//   start:   single exponential: the global minimum over a grid of rates by
//            variable projection (the oracle scans the same grid); double
//            exponential: the reference's initial guesses;
//   phase 1: FP32 Levenberg-Marquardt until the Gauss-Newton step is below
//            1e-4 sigma + 1e-6 |p| (or no step lowers chi^2);
//   phase 2: Newton with the full Hessian of chi^2/2 (J^T J - sum r d2f; the
//            Gauss-Newton matrix alone does not contract on these
//            large-residual problems), residuals and gradient in float-float
//            (the exponentials by a per-lane recurrence), to the least-squares
//            minimum: until the step is below 1e-9 sigma + 1e-12 |p|.
// ---------------------------------------------------------------------------

// u = (1 - e^{-kt}) / k and du/dk in FP32, x = k t >= 0 (ik = 1/k).
__device__ __forceinline__ void exp_u_f(float k, float ik, float t, float &u, float &dudk)
{
    const float x = k * t;
    if (fabsf(x) < 0.05f) {
        u = slow_exp_term(k, t);
        // du/dk = -t^2 (1/2 - x/3 + x^2/8 - x^3/30 + x^4/144)
        float d = fmaf(x, 1.f / 144.f, -1.f / 30.f);
        d = fmaf(x, d, 1.f / 8.f);
        d = fmaf(x, d, -1.f / 3.f);
        d = fmaf(x, d, 0.5f);
        dudk = -t * t * d;
    } else {
        const float em = (x < 0.7f) ? expm1f(-x) : __expf(-x) - 1.f;
        u = -em * ik;
        dudk = (t * (1.f + em) - u) * ik;
    }
}

// du/dk from an FP32 copy of e = e^{-kt} and u (series for small x).
__device__ __forceinline__ float exp_dudk(float k, float ik, float t, float e, float u)
{
    const float x = k * t;
    if (fabsf(x) < 0.05f) {
        float d = fmaf(x, 1.f / 144.f, -1.f / 30.f);
        d = fmaf(x, d, 1.f / 8.f);
        d = fmaf(x, d, -1.f / 3.f);
        d = fmaf(x, d, 0.5f);
        return -t * t * d;
    }
    return (t * e - u) * ik;
}

// (A + lambda diag(A) + ridge) x = b on the Jacobi-scaled system, FP32;
// parameters in `fix` (bit mask) are held: x_i = 0.
template <int K>
__device__ bool solve_scaled_k(const float *A, const float *b, float lambda, unsigned fix, float *x)
{
    float sc[K], L[K * K];
    for (int i = 0; i < K; i++) sc[i] = ((fix >> i) & 1) ? 0.f : rsqrtf(fmaxf(A[i * K + i], 1e-30f));
    for (int r = 0; r < K; r++)
        for (int c = 0; c < K; c++) L[r * K + c] = A[r * K + c] * sc[r] * sc[c];
    for (int i = 0; i < K; i++) L[i * K + i] = ((fix >> i) & 1) ? 1.f : 1.f + lambda + 1e-6f;
    for (int c = 0; c < K; c++) {
        float d = L[c * K + c];
        for (int m = 0; m < c; m++) d -= L[c * K + m] * L[c * K + m];
        if (!(d > 0.f) || !isfinite(d)) return false;
        d = sqrtf(d);
        L[c * K + c] = d;
        for (int r = c + 1; r < K; r++) {
            float s = L[r * K + c];
            for (int m = 0; m < c; m++) s -= L[r * K + m] * L[c * K + m];
            L[r * K + c] = s / d;
        }
    }
    float yv[K], z[K];
    for (int r = 0; r < K; r++) {
        float s = b[r] * sc[r];
        for (int m = 0; m < r; m++) s -= L[r * K + m] * yv[m];
        yv[r] = s / L[r * K + r];
    }
    for (int r = K - 1; r >= 0; r--) {
        float s = yv[r];
        for (int m = r + 1; m < K; m++) s -= L[m * K + r] * z[m];
        z[r] = s / L[r * K + r];
    }
    for (int r = 0; r < K; r++) x[r] = z[r] * sc[r];
    return true;
}

// d2u/dk2 of u = (1 - e^{-kt}) / k from e = e^{-kt} and u_k (series for
// small |x|, x = kt: t^3 (1/3 - x/4 + x^2/10 - x^3/36 + x^4/168)).
__device__ __forceinline__ float exp_d2udk2(float k, float ik, float t, float e, float uk)
{
    const float x = k * t;
    if (fabsf(x) < 0.05f) {
        float d = fmaf(x, 1.f / 168.f, -1.f / 36.f);
        d = fmaf(x, d, 0.1f);
        d = fmaf(x, d, -0.25f);
        d = fmaf(x, d, 1.f / 3.f);
        return t * t * t * d;
    }
    return (-t * t * e - 2.f * uk) * ik;
}

// One evaluation of the scaled model at p over the trace (warp).
//   precise = false: FP32 residuals, A = J^T J (Gauss-Newton matrix), g = J^T r;
//   precise = true:  residuals in float-float (the exponentials by a per-lane
//                    recurrence e <- e q seeded in FP64), A = the full Hessian
//                    of chi^2/2, J^T J - sum_i r_i d2f_i (FP32), g = J^T r
//                    accumulated in float-float and reduced in FP64.
// Returns chi^2 (float-float summed when precise).
template <int K>
__device__ __noinline__ double exp_normal(const float *y, int n, float dts, float iy, const double *p, bool precise,
                                          float *A, double *g, int lane)
{
    constexpr int NC = (K - 1) / 2;
    constexpr int NA = K * (K + 1) / 2;
    float acc[NA], gf[K];
    f2 gp[K];
    for (int i = 0; i < NA; i++) acc[i] = 0.f;
    for (int i = 0; i < K; i++) { gf[i] = 0.f; gp[i] = {0.f, 0.f}; }
    float pf[K], ik[NC];
    for (int i = 0; i < K; i++) pf[i] = (float)p[i];
    for (int c = 0; c < NC; c++) ik[c] = 1.f / pf[2 + 2 * c];
    f2 e[NC], q[NC], invk[NC], sp[NC], f0;
    bool slow[NC];
    if (precise) {
        f0 = f2_from_d(p[0]);
        for (int c = 0; c < NC; c++) {
            const double k = p[2 + 2 * c];
            e[c] = f2_from_d(exp(-k * ((double)lane + 0.5) * (double)dts));
            q[c] = f2_from_d(exp(-k * 32.0 * (double)dts));
            slow[c] = fabs(k * (double)n * (double)dts) < 1e-4;
            invk[c] = f2_from_d(slow[c] ? 0.0 : 1.0 / k);
            sp[c] = f2_from_d(p[1 + 2 * c]);
        }
    }
    float c2f = 0.f;            // FP32 phase: per-lane sum of ~n/32 squares
    f2 c2 = {0.f, 0.f};
    for (int x = lane; x < n; x += 32) {
        const float t = ((float)x + 0.5f) * dts;
        float gr[K], r;
        float hsk[NC], hkk[NC];   // d2f/(ds dk), d2f/dk2 per component (precise)
        gr[0] = 1.f;
        if (!precise) {
            float f = pf[0];
            for (int c = 0; c < NC; c++) {
                float u, du;
                exp_u_f(pf[2 + 2 * c], ik[c], t, u, du);
                f -= pf[1 + 2 * c] * u;
                gr[1 + 2 * c] = -u;
                gr[2 + 2 * c] = -pf[1 + 2 * c] * du;
            }
            r = __ldg(&y[x]) * iy - f;
            c2f = fmaf(r, r, c2f);
        } else {
            const f2 tf = f2_two_prod((float)x + 0.5f, dts);
            f2 f = f0;
            for (int c = 0; c < NC; c++) {
                f2 u;
                if (slow[c]) {
                    // u = t (1 - corr), corr = x/2 - x^2/6 + x^3/24 (|x| < 1e-4)
                    const float xx = pf[2 + 2 * c] * t;
                    const float corr = xx * (0.5f - xx * (1.f / 6.f - xx * (1.f / 24.f)));
                    u = f2_add(tf, f2_neg(f2_two_prod(tf.hi, corr)));
                } else {
                    u = f2_mul(f2_add({1.f, 0.f}, f2_neg(e[c])), invk[c]);
                }
                f = f2_add(f, f2_neg(f2_mul(sp[c], u)));
                const float uf = u.hi + u.lo, ef = e[c].hi + e[c].lo;
                const float uk = exp_dudk(pf[2 + 2 * c], ik[c], t, ef, uf);
                gr[1 + 2 * c] = -uf;
                gr[2 + 2 * c] = -pf[1 + 2 * c] * uk;
                hsk[c] = -uk;
                hkk[c] = -pf[1 + 2 * c] * exp_d2udk2(pf[2 + 2 * c], ik[c], t, ef, uk);
                e[c] = f2_mul(e[c], q[c]);
            }
            const f2 rr = f2_add(f2_two_prod(__ldg(&y[x]), iy), f2_neg(f));
            r = rr.hi + rr.lo;
            c2 = f2_add(c2, f2_mul(rr, rr));
            for (int a = 0; a < K; a++) gp[a] = f2_add(gp[a], f2_two_prod(gr[a], rr.hi));
            for (int a = 0; a < K; a++) gp[a] = f2_add(gp[a], f2_two_prod(gr[a], rr.lo));
        }
        int qa = 0;
        for (int a = 0; a < K; a++)
            for (int b = 0; b <= a; b++) acc[qa++] += gr[a] * gr[b];
        if (precise) {
            // - r d2f: the only nonzero second derivatives are (s_c, k_c) and (k_c, k_c)
            for (int c = 0; c < NC; c++) {
                const int is = 1 + 2 * c, ikk = 2 + 2 * c;
                acc[ikk * (ikk + 1) / 2 + is] -= r * hsk[c];
                acc[ikk * (ikk + 1) / 2 + ikk] -= r * hkk[c];
            }
        } else {
            for (int a = 0; a < K; a++) gf[a] += gr[a] * r;
        }
    }
    int qa = 0;
    for (int a = 0; a < K; a++)
        for (int b = 0; b <= a; b++) {
            float v = warp_sum(acc[qa++]);
            A[a * K + b] = v;
            A[b * K + a] = v;
        }
    for (int a = 0; a < K; a++)
        g[a] = precise ? warp_sum_d((double)gp[a].hi + (double)gp[a].lo) : (double)warp_sum(gf[a]);
    const double c2d = precise ? (double)c2.hi + (double)c2.lo : (double)c2f;
    return warp_sum_d(c2d);
}

// FP32 evaluation for phase 1 (no FP64 operation: GB300 issues FP64 at 1/64
// of the FP32 rate): chi^2, A = J^T J, g = J^T r at the FP32 parameters.
template <int K>
__device__ __noinline__ float exp_normal32(const float *y, int n, float dts, float iy, const float *pf, float *A,
                                           float *g, int lane)
{
    constexpr int NC = (K - 1) / 2;
    constexpr int NA = K * (K + 1) / 2;
    float acc[NA], gf[K], ik[NC];
    for (int i = 0; i < NA; i++) acc[i] = 0.f;
    for (int i = 0; i < K; i++) gf[i] = 0.f;
    for (int c = 0; c < NC; c++) ik[c] = 1.f / pf[2 + 2 * c];
    float c2f = 0.f;
    for (int x = lane; x < n; x += 32) {
        const float t = ((float)x + 0.5f) * dts;
        float gr[K];
        gr[0] = 1.f;
        float f = pf[0];
        for (int c = 0; c < NC; c++) {
            float u, du;
            exp_u_f(pf[2 + 2 * c], ik[c], t, u, du);
            f -= pf[1 + 2 * c] * u;
            gr[1 + 2 * c] = -u;
            gr[2 + 2 * c] = -pf[1 + 2 * c] * du;
        }
        const float r = __ldg(&y[x]) * iy - f;
        c2f = fmaf(r, r, c2f);
        int qa = 0;
        for (int a = 0; a < K; a++)
            for (int b = 0; b <= a; b++) acc[qa++] += gr[a] * gr[b];
        for (int a = 0; a < K; a++) gf[a] += gr[a] * r;
    }
    int qa = 0;
    for (int a = 0; a < K; a++)
        for (int b = 0; b <= a; b++) {
            const float v = warp_sum(acc[qa++]);
            A[a * K + b] = v;
            A[b * K + a] = v;
        }
    for (int a = 0; a < K; a++) g[a] = warp_sum(gf[a]);
    return warp_sum(c2f);
}

// FP32 counterpart of exp_newton_step (phase 1).
template <int K>
__device__ __forceinline__ bool exp_newton_step32(const float *A, const float *g, const float *p, unsigned &fix,
                                                  float *h)
{
    constexpr int NC = (K - 1) / 2;
    fix = 0;
    bool ok = solve_scaled_k<K>(A, g, 0.f, 0u, h);
    for (int c = 0; c < NC; c++)
        if (p[2 + 2 * c] <= 0.f && (!ok || h[2 + 2 * c] < 0.f)) fix |= 1u << (2 + 2 * c);
    if (fix) ok = solve_scaled_k<K>(A, g, 0.f, fix, h);
    return ok;
}

// The undamped (Gauss-)Newton step on A h = g, with a rate at its bound
// k = 0 held there (bit set in `fix`) when its step points below it.  The
// rate form is continuous through k = 0 (tau = infinity), so a trace whose
// minimum over k >= 0 is the linear limit reaches it exactly; the
// reference's A, tau, C cannot cross tau = infinity either and stop in that
// valley, on the k -> 0+ side.
template <int K>
__device__ __forceinline__ bool exp_newton_step(const float *A, const double *gd, const double *p, unsigned &fix,
                                                float *h)
{
    constexpr int NC = (K - 1) / 2;
    float g[K];
    for (int a = 0; a < K; a++) g[a] = (float)gd[a];
    fix = 0;
    bool ok = solve_scaled_k<K>(A, g, 0.f, 0u, h);
    for (int c = 0; c < NC; c++)
        if (p[2 + 2 * c] <= 0.0 && (!ok || h[2 + 2 * c] < 0.f)) fix |= 1u << (2 + 2 * c);
    if (fix) ok = solve_scaled_k<K>(A, g, 0.f, fix, h);
    return ok;
}

template <int K>
__global__ void bleach_exp_kernel(Job j, const float *trace, float *bp_out)
{
    constexpr int NC = (K - 1) / 2;
    const int lane = threadIdx.x & 31;
    const int tr = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (tr >= j.ntrace) return;
    const int n = j.nopit;
    const float *y = trace + (size_t)tr * n;
    const double dt_pt = (double)j.frametime * (double)j.ave;      // time per trace point (s)
    const float tmax = (float)(dt_pt * ((double)n - 0.5));
    const float dts = (float)(dt_pt / (double)tmax);               // scaled time per point
    float ym = 0.f;
    for (int x = lane; x < n; x += 32) ym = fmaxf(ym, fabsf(__ldg(&y[x])));
    for (int o = 16; o > 0; o >>= 1) ym = fmaxf(ym, __shfl_xor_sync(0xffffffffu, ym, o));
    if (ym == 0.f) ym = 1.f;
    const float iy = 1.f / ym;
    double p[K];
    if constexpr (K == 3) {
        // global search by variable projection: for each rate of the grid
        // x = k tmax in {0} and 96 log-spaced values 1e-3 .. 1e4 (the oracle's
        // grid), c0 + c1 e^{-kt} (k = 0: c0 + c1 t) is linear in c0, c1 and
        // chi^2 is minimised over them exactly; the best rate starts the LM
        float sy = 0.f;
        for (int x = lane; x < n; x += 32) sy += __ldg(&y[x]) * iy;
        const float my = warp_sum(sy) / (float)n;
        float syy = 0.f;
        for (int x = lane; x < n; x += 32) { const float yc = __ldg(&y[x]) * iy - my; syy = fmaf(yc, yc, syy); }
        syy = warp_sum(syy);
        // eight rates per pass over the trace: independent recurrences and
        // reductions overlap (the per-rate sums are those of one rate at a
        // time, so the choice is the same)
        constexpr int RB = 8;
        float bc = 3.4e38f, b0 = 0.f, b1 = 0.f, bk = 0.f;
        for (int jb = 0; jb < 97; jb += RB) {
            float kx[RB], q[RB], e0[RB], se[RB], e[RB];
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const int jg = jb + r;
                kx[r] = (jg == 0 || jg > 96) ? 0.f : exp10f(-3.f + 7.f * (float)(jg - 1) / 95.f);
                q[r] = __expf(-kx[r] * 32.f * dts);
                e0[r] = __expf(-kx[r] * ((float)lane + 0.5f) * dts);
                se[r] = 0.f;
                e[r] = e0[r];
            }
            for (int x = lane; x < n; x += 32) {
                const float tt = ((float)x + 0.5f) * dts;
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    se[r] += (jb + r == 0) ? tt : e[r];
                    e[r] *= q[r];
                }
            }
            float me[RB], see[RB], sye[RB];
#pragma unroll
            for (int r = 0; r < RB; r++) {
                me[r] = warp_sum(se[r]) / (float)n;
                see[r] = 0.f;
                sye[r] = 0.f;
                e[r] = e0[r];
            }
            for (int x = lane; x < n; x += 32) {
                const float tt = ((float)x + 0.5f) * dts;
                const float yc = __ldg(&y[x]) * iy - my;
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    const float b = ((jb + r == 0) ? tt : e[r]) - me[r];
                    see[r] = fmaf(b, b, see[r]);
                    sye[r] = fmaf(yc, b, sye[r]);
                    e[r] *= q[r];
                }
            }
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const float sE = warp_sum(see[r]), sY = warp_sum(sye[r]);
                if (jb + r > 96) continue;
                const float c1 = sE > 0.f ? sY / sE : 0.f;
                const float c2 = syy - c1 * sY;
                if (c2 < bc) { bc = c2; b1 = c1; b0 = my - c1 * me[r]; bk = kx[r]; }
            }
        }
        if (bk == 0.f) { p[0] = b0; p[1] = -b1; p[2] = 0.0; }                  // f = c0 + c1 t
        else { p[0] = (double)b0 + b1; p[1] = (double)b1 * bk; p[2] = bk; }       // f = c0 + c1 e^{-kt}
    } else {
        // reference initial guesses (java:10917-10921) in f0, s, k
        const double y1 = (double)__ldg(&y[1]) * (double)iy;
        const double thalf = ((double)(n / 2) + 0.5) * (double)dts;
        {
            const double t10 = ((double)(n / 10) + 0.5) * (double)dts;
            p[0] = y1; p[1] = 0.5 * y1 / t10; p[2] = 1.0 / t10; p[3] = 0.5 * y1 / thalf; p[4] = 1.0 / thalf;
        }
    }
    // Phase 1: FP32 Levenberg-Marquardt (FP32 parameters, no FP64 operation)
    // until the Gauss-Newton step is below 1e-3 sigma + 1e-6 |p| (or, with
    // that step within 0.05 sigma, two steps in a row fail to lower chi^2,
    // or no step lowers it up to lambda 1e10): inside the region where the Newton
    // phase converges quadratically; FP32 sums over 1000 points cannot
    // resolve much smaller steps anyway.
    float A[K * K], lambda = 1e-3f;
    double g[K];
    float pf[K], gf[K];
    for (int a = 0; a < K; a++) pf[a] = (float)p[a];
    float chi2f = exp_normal32<K>(y, n, dts, iy, pf, A, gf, lane);
    const bool ok = isfinite(chi2f);
    int evals = 1, rejected = 0;
    for (int it_n = 0; ok && it_n < 100; it_n++) {
        float h[K];
        unsigned fix;
        bool gn_near = false;      // Gauss-Newton step within 0.05 sigma
        if (exp_newton_step32<K>(A, gf, pf, fix, h)) {
            bool conv = true;
            gn_near = true;
            for (int a = 0; a < K; a++) {
                if ((fix >> a) & 1) continue;
                const float sig = rsqrtf(fmaxf(A[a * K + a], 1e-30f));
                conv = conv && fabsf(h[a]) <= 1e-6f * fabsf(pf[a]) + 1e-3f * sig;
                gn_near = gn_near && fabsf(h[a]) <= 0.05f * sig;
            }
            if (conv) break;
        }
        if (!solve_scaled_k<K>(A, gf, lambda, fix, h)) {
            lambda *= 10.f;
            if (lambda > 1e10f) break;
            continue;
        }
        float pn[K];
        for (int a = 0; a < K; a++) pn[a] = pf[a] + h[a];
        for (int c = 0; c < NC; c++) pn[2 + 2 * c] = fmaxf(pn[2 + 2 * c], 0.f);
        float An[K * K], gn[K];
        const float c2n = exp_normal32<K>(y, n, dts, iy, pn, An, gn, lane);
        evals++;
        if (isfinite(c2n) && c2n < chi2f) {
            for (int a = 0; a < K; a++) { pf[a] = pn[a]; gf[a] = gn[a]; }
            for (int a = 0; a < K * K; a++) A[a] = An[a];
            chi2f = c2n;
            lambda = fmaxf(lambda * 0.1f, 1e-12f);
            rejected = 0;
        } else {
            // two rejected steps in a row while the Gauss-Newton step is
            // within 0.05 sigma: FP32 chi^2 no longer resolves the descent
            // this close to the minimum -- the Newton phase takes over
            // (elsewhere rejections raise the damping as usual)
            rejected = gn_near ? rejected + 1 : 0;
            lambda *= 10.f;
            if (lambda > 1e10f || rejected >= 2) break;
        }
    }
    for (int a = 0; a < K; a++) p[a] = (double)pf[a];
    double chi2 = chi2f;
    // Phase 2: Newton with the full Hessian, float-float residuals and
    // gradient, to the least-squares minimum: until the step is below
    // 1e-9 sigma + 1e-12 |p|, while chi^2 does not increase.
    if (ok) {
        chi2 = exp_normal<K>(y, n, dts, iy, p, true, A, g, lane);
        evals++;
        for (int it_n = 0; it_n < 20 && isfinite(chi2); it_n++) {
            float h[K];
            unsigned fix;
            if (!exp_newton_step<K>(A, g, p, fix, h)) break;   // Hessian not positive definite
            bool conv = true;
            for (int a = 0; a < K; a++) {
                if ((fix >> a) & 1) continue;
                const float sig = rsqrtf(fmaxf(A[a * K + a], 1e-30f));
                conv = conv && fabsf(h[a]) <= 1e-12f * (float)fabs(p[a]) + 1e-9f * sig;
            }
            double pn[K];
            for (int a = 0; a < K; a++) pn[a] = p[a] + (double)h[a];
            for (int c = 0; c < NC; c++) pn[2 + 2 * c] = fmax(pn[2 + 2 * c], 0.0);
            float An[K * K];
            double gn[K];
            const double c2n = exp_normal<K>(y, n, dts, iy, pn, true, An, gn, lane);
            evals++;
            if (!(isfinite(c2n) && c2n <= chi2)) break;
            for (int a = 0; a < K; a++) { p[a] = pn[a]; g[a] = gn[a]; }
            for (int a = 0; a < K * K; a++) A[a] = An[a];
            chi2 = c2n;
            if (conv) break;
        }
    }
    // back to data units: y = y_s / iy, t = t_s tmax
    const double st = (double)dts / dt_pt;            // 1 / tmax
    const double f0d = p[0] / (double)iy;
    double sd[NC], kd[NC];
    bool valid = ok && isfinite(f0d);
    for (int c = 0; c < NC; c++) {
        sd[c] = p[1 + 2 * c] * st / (double)iy;
        kd[c] = p[2 + 2 * c] * st;
        valid = valid && isfinite(sd[c]) && isfinite(kd[c]) && sd[c] != 0.0;  // java:9689, 9714
    }
    // curve evaluation form per component (exp form unless slow over the run)
    const double t_end = (double)j.frametime * ((double)j.num + 2.0);
    float bpl[kBleachStride];
    for (int a = 0; a < kBleachStride; a++) bpl[a] = 0.f;
    double cconst = f0d, csum_amp = 0.0;
    int flags = 0;
    for (int c = 0; c < NC; c++) {
        const double amp = sd[c] / kd[c];               // A_c (inf when k_c = 0)
        bpl[5 + c] = (float)kd[c];
        if (fabs(kd[c]) * t_end <= 0.5) {
            flags |= 1 << c;
            bpl[7 + c] = (float)sd[c];
        } else {
            bpl[7 + c] = (float)amp;
            cconst -= amp;
        }
        csum_amp += amp;
        // reference form: A_c, tau_c
        bpl[2 * c] = (float)amp;
        bpl[2 * c + 1] = (float)(1.0 / kd[c]);
    }
    bpl[2 * NC] = (float)(f0d - csum_amp);               // C
    bpl[13] = (float)cconst;
    bpl[14] = (float)flags;
    const float f0 = (float)f0d, inv_f0 = (float)(1.0 / f0d);
    float csum = 0.f, cnt = 0.f;     // centre over the finite corrected points
    for (int x = lane; x < n; x += 32) {
        float yx = __ldg(&y[x]);
        if (valid) {
            float t = j.frametime * ((float)x + 0.5f) * (float)j.ave;
            yx = bleach_correct(yx, bleach_f(bpl, j.bleach, 0, t, nullptr), f0, inv_f0);
        }
        if (isfinite(yx)) { csum += yx; cnt += 1.f; }
    }
    csum = warp_sum(csum);
    cnt = warp_sum(cnt);
    if (lane == 0) {
        float *bp = bp_out + (size_t)tr * kBleachStride;
        for (int a = 0; a < kBleachStride; a++) bp[a] = bpl[a];
        bp[9] = f0;
        bp[10] = inv_f0;
        bp[11] = valid ? 1.f : 0.f;
        bp[12] = cnt > 0.f ? csum / cnt : 0.f;
        bp[15] = (float)evals;      // model evaluations (diagnostic)
    }
}

// Finalise monitors: one warp per output pixel.  Exclusive scan of the
// segment totals (FP64), snapshot prefixes, then for every lag
//   a = sum(direct window)/n - 2^k c0,  b = sum(delayed window)/n - 2^k c1,
// dm = a + 2^k c0, Dm = b + 2^k c1  (java:9484-9491), plus the lag-1 monitors
// of the zero-led sequence blockTransform reads (java:9259-9272).
//
// Non-finite corrected frames entered the sums as 0 and are counted; a
// window that contains one gives a NaN monitor, so exactly the lags whose
// windows hold a bad frame become non-finite, as calculateCF's sums do
// (java:9484-9491).
__global__ void monitor_finalize_kernel(Job j, const LagInfo *li, const float *bparams,
                                        int nseg, const float2 *segtot, const float2 *snap_part,
                                        const int *segbad, const int *snap_bad, float4 *mon, float4 *blkmon)
{
    extern __shared__ double sh[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int pix = blockIdx.x * (blockDim.x >> 5) + wid;
    if (pix >= j.npix) return;
    double *scan = sh + (size_t)wid * (nseg + 1 + 4 * j.nsnap);
    double *pre0 = scan + nseg + 1;
    double *pre1 = pre0 + j.nsnap;
    double *bad0 = pre1 + j.nsnap;      // prefix counts of non-finite frames
    double *bad1 = bad0 + j.nsnap;
    for (int which = 0; which < (j.is_ccf ? 2 : 1); which++) {
        int tr = which ? j.npix + pix : pix;
        double *pre = which ? pre1 : pre0;
        double *bpre = which ? bad1 : bad0;
        // exclusive scans of the segment totals (pass 0) and of the
        // non-finite frame counts (pass 1), then the snapshot prefixes
        for (int pass = 0; pass < 2; pass++) {
            double carry = 0.0;
            for (int s0 = 0; s0 < nseg; s0 += 32) {
                int s = s0 + lane;
                double v = 0.0;
                if (s < nseg) {
                    if (pass == 0) { float2 t = segtot[(size_t)tr * nseg + s]; v = (double)t.x + (double)t.y; }
                    else v = (double)segbad[(size_t)tr * nseg + s];
                }
                double incl = v;
                for (int o = 1; o < 32; o <<= 1) {
                    double u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += u;
                }
                if (s < nseg) scan[s] = carry + incl - v;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (lane == 0) scan[nseg] = carry;
            __syncwarp();
            for (int sj = lane; sj < j.nsnap; sj += 32) {
                int p = li->snap_pos[sj];
                double v = 0.0;
                if (p > 0) {
                    int seg = (p - 1) / kSeg;
                    if (pass == 0) {
                        float2 t = snap_part[(size_t)tr * j.nsnap + sj];
                        v = scan[seg] + (double)t.x + (double)t.y;
                    } else {
                        v = scan[seg] + (double)snap_bad[(size_t)tr * j.nsnap + sj];
                    }
                }
                (pass == 0 ? pre : bpre)[sj] = v;
            }
            __syncwarp();
        }
    }
    if (!j.is_ccf)
        for (int sj = lane; sj < j.nsnap; sj += 32) { pre1[sj] = pre0[sj]; bad1[sj] = bad0[sj]; }
    __syncwarp();
    const double c0 = bparams[(size_t)pix * kBleachStride + 12];
    const double c1 = bparams[(size_t)(j.is_ccf ? j.npix + pix : pix) * kBleachStride + 12];
    for (int x = lane; x < j.chanum; x += 32) {
        int k = li->level[x];
        double n = li->prodnum[x];
        double a = pre0[li->snap_dir_end[x]] / n;
        double b = (pre1[li->snap_del_end[x]] - pre1[li->snap_del_beg[x]]) / n;
        if (bad0[li->snap_dir_end[x]] > 0.0) a = nan("");
        if (bad1[li->snap_del_end[x]] - bad1[li->snap_del_beg[x]] > 0.0) b = nan("");
        double sc = (double)(1 << k);
        mon[(size_t)pix * j.chanum + x] =
            make_float4((float)a, (float)b, (float)(a + sc * c0), (float)(b + sc * c1));
    }
    if (lane == 0) {
        double T1 = j.num - 1;
        double dm1 = (pre0[li->snap_tm2] + (j.num - 2) * c0) / T1;   // zero-led direct window
        double Dm1 = (pre1[li->snap_tm1] + (j.num - 1) * c1) / T1;
        if (bad0[li->snap_tm2] > 0.0) dm1 = nan("");
        if (bad1[li->snap_tm1] > 0.0) Dm1 = nan("");
        blkmon[pix] = make_float4((float)(dm1 - c0), (float)(Dm1 - c1), (float)dm1, (float)Dm1);
    }
}

// ---------------------------------------------------------------------------
// Blocking pass (blockTransform, java:9217-9422).  The lag-1 products of the
// zero-led sequence J = [0, v_0, ..., v_{T-2}] are
//   p_j = (J_j - dm1) (J_{j+1} - Dm1),  j = 0 .. T-2,
// blocked pairwise (block means, java:9308-9316).  One thread per (pixel,
// segment of 256 products) computes, for levels 0..8, the sums of block means
// and squared block means of the complete blocks inside its segment, and the
// segment sum for the higher levels.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) block_kernel(Job j, const float *s0a, const float *s0b,
                                                    const float4 *blkmon, int nbseg, float *s1, float *s2,
                                                    float *segsum)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    const int seg = blockIdx.y;
    if (pix >= j.npix) return;
    const float *sb = j.is_ccf ? s0b : s0a;
    const float4 bm = blkmon[pix];   // a1 = dm1 - c0, b1 = Dm1 - c1, dm1, Dm1
    const int nprod = j.num - 1;
    const int j0 = seg * kBlkSeg, j1 = min(j0 + kBlkSeg, nprod);
    float S1[kBlkSegLog + 1], S2[kBlkSegLog + 1], pend[kBlkSegLog + 1];
#pragma unroll
    for (int y = 0; y <= kBlkSegLog; y++) { S1[y] = 0.f; S2[y] = 0.f; pend[y] = 0.f; }
    // direct element of product jj is J_jj = v_{jj-1} (J_0 = 0); s0 holds the
    // corrected values centred on c, so J - dm1 = s0 - (dm1 - c)
    float u_prev = (j0 == 0) ? -bm.z : __ldg(&s0a[(size_t)(j0 - 1) * j.npix + pix]) - bm.x;
    float segv = 0.f;
    for (int tb = j0; tb < j1; tb += 8) {
        float va[8], vb[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const bool in = tb + u < j1;
            va[u] = in ? __ldg(&s0a[(size_t)(tb + u) * j.npix + pix]) : 0.f;
            vb[u] = (in && j.is_ccf) ? __ldg(&sb[(size_t)(tb + u) * j.npix + pix]) : va[u];
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int jj = tb + u;
            if (jj >= j1) break;
            const float w = vb[u] - bm.y;
            const float p = u_prev * w;
            u_prev = va[u] - bm.x;   // next direct element J_{jj+1} = v_jj
            const int rel = jj - j0;
            S1[0] += p;
            S2[0] += p * p;
            // pairwise block means: level y+1 completes when bit y of rel is
            // set; unrolled so that every array index is a constant (registers)
            float v = p;
            bool carry = true;
#pragma unroll
            for (int y = 0; y < kBlkSegLog; y++) {
                if (carry) {
                    if ((rel >> y) & 1) {
                        v = pend[y] + v;
                        const float m = v * (1.f / (float)(1 << (y + 1)));
                        S1[y + 1] += m;
                        S2[y + 1] += m * m;
                    } else {
                        pend[y] = v;
                        carry = false;
                    }
                }
            }
            if (carry) segv = v;
        }
    }
    // [level][segment][pixel]: coalesced here and in the finaliser
#pragma unroll
    for (int y = 0; y <= kBlkSegLog; y++) {
        const size_t o = ((size_t)y * nbseg + seg) * j.npix + pix;
        s1[o] = S1[y];
        s2[o] = S2[y];
    }
    segsum[(size_t)seg * j.npix + pix] = segv;     // used only for complete segments
}

// Blocking decision.  A CTA serves 32 pixels with 8 threads each: thread
// (pixel, t) sums the segments' statistics of levels t, t + 8, ... in FP64
// (coalesced across pixels; each level's sum in segment order), the levels
// above the segment size from segment sums; then one thread per pixel
// applies the overlap / monotonic-increase criteria of java:9339-9380.
constexpr int kBlkFinPix = 32, kBlkFinLev = 8;
__global__ void __launch_bounds__(kBlkFinPix * kBlkFinLev)
block_finalize_kernel(Job j, int q, int nbseg, const float *s1, const float *s2, const float *segsum,
                      const float4 *blkmon, int *ind_out, int *ok_out)
{
    __shared__ double S1s[kMaxBlockLevels][kBlkFinPix], S2s[kMaxBlockLevels][kBlkFinPix];
    const int pl = threadIdx.x % kBlkFinPix, ty = threadIdx.x / kBlkFinPix;
    const int pix = blockIdx.x * kBlkFinPix + pl;
    const int blocknum = j.blocknum;
    const int full_segs = (j.num - 1) / kBlkSeg;   // segments holding kBlkSeg products
    if (pix < j.npix) {
        for (int y = ty; y < blocknum; y += kBlkFinLev) {
            double a1 = 0.0, a2 = 0.0;
            if (y <= kBlkSegLog) {
                const float *p1 = s1 + (size_t)y * nbseg * j.npix + pix, *p2 = s2 + (size_t)y * nbseg * j.npix + pix;
                for (int seg = 0; seg < nbseg; seg++) {
                    a1 += (double)__ldg(&p1[(size_t)seg * j.npix]);
                    a2 += (double)__ldg(&p2[(size_t)seg * j.npix]);
                }
            } else {
                // levels above the segment: block y spans 2^(y-8) consecutive
                // complete segments (a non-finite segment sum, from a
                // non-finite frame, propagates like the Java sums)
                const int span = 1 << (y - kBlkSegLog);
                const double inv = 1.0 / (double)(1 << y);
                for (int b = 0; (b + 1) * span <= full_segs; b++) {
                    double sb = 0.0;
                    for (int k = 0; k < span; k++) sb += (double)__ldg(&segsum[(size_t)(b * span + k) * j.npix + pix]);
                    const double m = sb * inv;
                    a1 += m;
                    a2 += m * m;
                }
            }
            S1s[y][pl] = a1;
            S2s[y][pl] = a2;
        }
    }
    __syncthreads();
    if (ty != 0 || pix >= j.npix) return;
    double S1[kMaxBlockLevels], S2[kMaxBlockLevels];
    for (int y = 0; y < blocknum; y++) {
        S1[y] = S1s[y][pl];
        S2[y] = S2s[y][pl];
    }
    const float4 bm = blkmon[pix];
    const double dmDm = (double)bm.z * (double)bm.w;
    const int nprod = j.num - 1;
    double vb1[kMaxBlockLevels], upper[kMaxBlockLevels], lower[kMaxBlockLevels];
    int crt[kMaxBlockLevels] = {0}, cr12[kMaxBlockLevels] = {0}, cr3[kMaxBlockLevels] = {0},
        diffpos[kMaxBlockLevels] = {0};
    for (int y = 0; y < blocknum; y++) {
        double n = (double)(nprod >> y);
        double v = (S2[y] / n - (S1[y] / n) * (S1[y] / n)) / (n * dmDm * dmDm);
        vb1[y] = sqrt(v);
        double e = vb1[y] / sqrt(2 * (n - 1));
        upper[y] = vb1[y] + e;
        lower[y] = vb1[y] - e;
    }
    for (int x = 0; x < blocknum - 1; x++)
        if (upper[x] > lower[x + 1] && upper[x + 1] > lower[x]) crt[x] = 1;
    for (int x = 0; x < blocknum - 2; x++)
        if (crt[x] * crt[x + 1] == 1) cr12[x] = 1;
    for (int x = 0; x < blocknum - 1; x++)
        if (vb1[x + 1] - vb1[x] > 0) diffpos[x] = 1;
    for (int x = 0; x < blocknum - 2; x++)
        if (diffpos[x] * diffpos[x + 1] == 1) cr3[x] = 1;
    int last0 = 0;
    for (int x = 0; x < blocknum - 2; x++)
        if (cr3[x] == 1 && cr12[x] == 0) last0 = x;
    for (int x = 0; x <= last0; x++) cr12[x] = 0;
    if (blocknum >= 3) cr12[blocknum - 3] = 0;
    if (blocknum >= 4) cr12[blocknum - 4] = 0;
    int ind = 0, ok;
    for (int x = blocknum - 5; x > 0; x--)
        if (cr12[x] == 1) ind = x + 1;
    if (ind == 0) {
        ok = 0;
        ind = (blocknum - 3 > 0) ? blocknum - 3 : blocknum - 1;
    } else {
        ok = 1;
    }
    if (ind < q - 1) ind = q - 1;
    ind_out[pix] = ind;
    ok_out[pix] = ok;
}

// Centre of traces whose bleach parameters were supplied by the caller
// (reference calcACF path): mean of the corrected averaged trace.
__global__ void center_given_kernel(Job j, const float *trace, float *bp_out)
{
    const int lane = threadIdx.x & 31;
    const int tr = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (tr >= j.ntrace) return;
    float *bp = bp_out + (size_t)tr * kBleachStride;
    const float *y = trace + (size_t)tr * j.nopit;
    float bpl[kBleachStride];
    for (int i = 0; i < kBleachStride; i++) bpl[i] = bp[i];
    float s = 0.f, cnt = 0.f, lb[kMaxPoly + 1];
    for (int x = lane; x < j.nopit; x += 32) {
        float v = __ldg(&y[x]);
        if (j.bleach != IMFCS_BLEACH_NONE && bpl[11] != 0.f) {
            float t = j.frametime * ((float)x + 0.5f) * (float)j.ave;
            if (j.bleach == IMFCS_BLEACH_POLYNOMIAL) legendre(t * bpl[13] + bpl[14], j.poly_order, lb);
            v = bleach_correct(v, bleach_f(bpl, j.bleach, j.poly_order, t, lb), bpl[9], bpl[10]);
        }
        if (isfinite(v)) { s += v; cnt += 1.f; }
    }
    s = warp_sum(s);
    cnt = warp_sum(cnt);
    if (lane == 0) bp[12] = cnt > 0.f ? s / cnt : 0.f;
}

// Stride-1 box-sum binning of a float stack (calc_binning, agpufitjni.cu:4560-4586).
__global__ void binning_kernel(const float *in, float *out, int win, int hin, int wt, int ht,
                               int frames, int bx, int by)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)wt * ht * frames;
    if (i >= n) return;
    int x = (int)(i % wt);
    int y = (int)((i / wt) % ht);
    size_t t = i / ((size_t)wt * ht);
    const float *f = in + t * (size_t)win * hin;
    float s = 0.f;
    for (int a = 0; a < bx; a++)
        for (int b = 0; b < by; b++) s += f[(size_t)(y + b) * win + x + a];
    out[i] = s;
}

// Averages of `ave` frames per pixel of a float stack [t][h][w] -> [h][w][nopit]
// with the Java CPU's truncating division (java:9852).
__global__ void bleach_average_kernel(const float *in, float *out, int w, int h, int nopit, int ave)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)w * h * nopit) return;
    int pix = (int)(i / nopit), x = (int)(i % nopit);
    double s = 0.0;
    for (int f = x * ave; f < (x + 1) * ave; f++) s += in[(size_t)f * w * h + pix];
    out[i] = (float)trunc(s / ave);
}

// Explicit instantiations used by the host side.
template __global__ void bleach_exp_kernel<3>(Job, const float *, float *);
template __global__ void bleach_exp_kernel<5>(Job, const float *, float *);

}  // namespace imfcs

namespace imfcs {

cudaError_t launch_trace(const Job &j, const void *stack, float *trace, cudaStream_t s)
{
    dim3 grid((j.ntrace + 31) / 32, (j.nopit + 31) / 32), block(32, 8);
    trace_kernel<<<grid, block, 0, s>>>(j, stack, trace);
    return cudaGetLastError();
}

cudaError_t launch_bleach(const Job &j, const float *trace, const double *proj, float uscale,
                          float uoff, float *bparams, cudaStream_t s)
{
    const int threads = 128;
    const int blocks = (j.ntrace * 32 + threads - 1) / threads;
    switch (j.bleach) {
    case IMFCS_BLEACH_POLYNOMIAL:
        bleach_poly_kernel<<<blocks, threads, 0, s>>>(j, trace, proj, uscale, uoff, bparams);
        break;
    case IMFCS_BLEACH_SINGLE_EXP:
        bleach_exp_kernel<3><<<blocks, threads, 0, s>>>(j, trace, bparams);
        break;
    case IMFCS_BLEACH_DOUBLE_EXP:
        bleach_exp_kernel<5><<<blocks, threads, 0, s>>>(j, trace, bparams);
        break;
    default:
        center_kernel<<<blocks, threads, 0, s>>>(j, trace, bparams);
    }
    return cudaGetLastError();
}

cudaError_t launch_center_given(const Job &j, const float *trace, float *bparams, cudaStream_t s)
{
    const int threads = 128;
    center_given_kernel<<<(j.ntrace * 32 + threads - 1) / threads, threads, 0, s>>>(j, trace, bparams);
    return cudaGetLastError();
}

cudaError_t launch_monitor_finalize(const Job &j, const LagInfo *li_dev, const float *bparams, int nseg,
                                    const float2 *segtot, const float2 *snap_part, const int *segbad,
                                    const int *snap_bad, float4 *mon, float4 *blkmon, cudaStream_t s)
{
    const int wpb = 4;
    size_t smem = (size_t)wpb * (nseg + 1 + 4 * j.nsnap) * sizeof(double);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(monitor_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    monitor_finalize_kernel<<<(j.npix + wpb - 1) / wpb, wpb * 32, smem, s>>>(j, li_dev, bparams, nseg, segtot,
                                                                           snap_part, segbad, snap_bad, mon,
                                                                           blkmon);
    return cudaGetLastError();
}

cudaError_t launch_block(const Job &j, const float *s0, const float4 *blkmon, int nbseg, float *s1, float *s2,
                         float *segsum, int *ind, int *ok, cudaStream_t s)
{
    dim3 grid((j.npix + 127) / 128, nbseg);
    const float *s0b = j.is_ccf ? s0 + (size_t)j.npix * j.num : s0;
    block_kernel<<<grid, 128, 0, s>>>(j, s0, s0b, blkmon, nbseg, s1, s2, segsum);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    block_finalize_kernel<<<(j.npix + kBlkFinPix - 1) / kBlkFinPix, kBlkFinPix * kBlkFinLev, 0, s>>>(
        j, j.q, nbseg, s1, s2, segsum, blkmon, ind, ok);
    return cudaGetLastError();
}

cudaError_t launch_binning(const float *in, float *out, int win, int hin, int wt, int ht,
                           int frames, int bx, int by, cudaStream_t s)
{
    size_t n = (size_t)wt * ht * frames;
    binning_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, win, hin, wt, ht, frames, bx, by);
    return cudaGetLastError();
}

cudaError_t launch_bleach_average(const float *in, float *out, int w, int h, int nopit, int ave,
                                  cudaStream_t s)
{
    size_t n = (size_t)w * h * nopit;
    bleach_average_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, w, h, nopit, ave);
    return cudaGetLastError();
}

}  // namespace imfcs
