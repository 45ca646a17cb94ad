// imfcs_internal.cuh -- shared device/host definitions of the GB300 engine.
//
// Data layout in HBM
//   stack      uint16 [frames][height][width]   (as acquired; read-only)
//              or float [frames][h_temp][w_temp] for the reference calcACF path
//   traces     a "trace" is one binned, background-subtracted pixel window;
//              trace t < npix is the direct window of output pixel t, trace
//              npix + t its displaced window (spatial cross-correlation).
//   per-trace  scratch is [trace][...] (pixel-major), per-lag results are
//              [pixel][lag].
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "imfcs_gb300.h"

namespace imfcs {

constexpr int kMaxChan = 160;      // chanum limit (P = 16 -> Q <= 18)
constexpr int kMaxLevels = 16;     // correlator levels (Q)
constexpr int kMaxBlockLevels = 32;
constexpr int kMaxSnap = 3 * kMaxChan + 8;
constexpr int kTile = 32;          // output pixels per correlator CTA (one warp lane each)
constexpr int kChunk = 128;        // frames staged per correlator step
constexpr int kP = 16;             // correlator P of the level chain (P = 32: the generic level kernel)
constexpr int kHist = kP;          // window history kept per level
constexpr int kMaxPoly = 8;        // polynomial bleach order (java BCmaxorder = 8)
constexpr int kBleachStride = 16;  // floats per trace in the bleach-parameter array
constexpr int kSeg = 256;          // frames per monitor segment
constexpr int kBlkSeg = 256;       // products per blocking segment (2^8)
constexpr int kBlkSegLog = 8;

// Job descriptor passed by value to kernels (all sizes derived on the host).
struct Job {
    // input geometry
    int in_w, in_h;               // input frame geometry
    int input_float;              // 0: uint16 raw stack, 1: float stack
    int first, num;               // first frame (0-based) and frame count
    int out_w, out_h, map_x0, map_y0;
    int binx, biny, pixbinx, pixbiny;
    int cfx, cfy;
    int background;
    // per-pixel background image (java:9671-9673, 9842-9845): per-trace sums
    // of the rounded image over the trace's window for its values, and over
    // the direct window for its averaged trace; nullptr = scalar background
    const int *bg_trace;
    const int *bg_avg;
    int is_ccf;
    int npix, ntrace;
    // correlator structure
    int p, q, chanum;
    int nopit, ave;
    float frametime;
    double frametime_d;
    int bleach, poly_order;
    int blocknum;                 // floor(log2(mtab[1])) - 2
    // lag tables (device copies live in constant memory per launch via Job)
    int nsnap;
    // correlator tile of the level chain (chosen by the autotuner): pixels
    // per CTA (32 or 64; 0 = 64) and frame segments of the pair kernels and
    // of the tail kernel, 2^c2_seg_extra and 2^c2_tail_extra times the
    // shortest legal segment
    int c2_cta, c2_seg_extra, c2_tail_extra;
};

// Lag tables, snapshot positions and per-lag snapshot indices, stored in a
// small device buffer and copied into shared memory by kernels that need
// them.
struct LagInfo {
    int lag[kMaxChan];
    int level[kMaxChan];          // log2(samp)
    int del[kMaxChan];            // lag / samp
    int prodnum[kMaxChan];        // numbin_k - del
    int snap_dir_end[kMaxChan];   // snapshot index of prodnum * 2^k
    int snap_del_beg[kMaxChan];   // snapshot index of lag
    int snap_del_end[kMaxChan];   // snapshot index of numbin_k * 2^k
    int snap_pos[kMaxSnap];       // sorted unique snapshot positions (frames)
    int snap_tm2, snap_tm1;       // snapshot indices of num-2 and num-1
    int numbin[kMaxLevels];
    int nlevels;
    int pnum_by_ind[kMaxBlockLevels];  // pnum for each possible block index
    int nsnap;
};

// ---------------------------------------------------------------------------
// Float-float (double-single) accumulation: exact two-sum (Knuth).
// ---------------------------------------------------------------------------
struct ff {
    float hi, lo;
};
__device__ __forceinline__ void ff_add(ff &a, float b)
{
    float s = __fadd_rn(a.hi, b);
    float bb = __fsub_rn(s, a.hi);
    float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, err);
}
__device__ __forceinline__ double ff_val(const ff &a) { return (double)a.hi + (double)a.lo; }

// ---------------------------------------------------------------------------
// Window value of one trace at frame t (0-based, relative to job.first).
// ---------------------------------------------------------------------------
// Background subtracted from trace `trace`'s window sum (its values), and
// from the window sums of its averaged trace.
__device__ __forceinline__ int trace_bg(const Job &j, int trace)
{
    return j.bg_trace ? __ldg(&j.bg_trace[trace]) : j.background * j.binx * j.biny;
}
__device__ __forceinline__ int trace_bg_avg(const Job &j, int trace)
{
    return j.bg_avg ? __ldg(&j.bg_avg[trace]) : j.background * j.binx * j.biny;
}

// bg: the window's background sum (uint16 input; the float input arrives
// background-subtracted).
__device__ __forceinline__ float window_value(const Job &j, const void *stack, int x0, int y0,
                                              int t, int bg)
{
    const size_t fsz = (size_t)j.in_w * j.in_h;
    const size_t base = (size_t)(j.first + t) * fsz;
    if (!j.input_float) {
        const uint16_t *s = (const uint16_t *)stack + base;
        int acc = 0;
        for (int k = 0; k < j.biny; k++)
            for (int i = 0; i < j.binx; i++)
                acc += (int)__ldg(&s[(size_t)(y0 + k) * j.in_w + x0 + i]);
        return (float)(acc - bg);
    } else {
        const float *s = (const float *)stack + base;
        float acc = 0.f;
        for (int k = 0; k < j.biny; k++)
            for (int i = 0; i < j.binx; i++) acc += __ldg(&s[(size_t)(y0 + k) * j.in_w + x0 + i]);
        return acc;
    }
}

// N consecutive frames t..t+N-1 of one window (frames >= tmax read as 0).
// The loads are issued back to back so that a thread keeps N requests in
// flight (the streaming passes are latency-bound otherwise).
template <int N>
__device__ __forceinline__ void window_values(const Job &j, const void *stack, int x0, int y0, int t,
                                              int tmax, int bg, float *v)
{
    const size_t fsz = (size_t)j.in_w * j.in_h;
    if (!j.input_float && j.binx == 1 && j.biny == 1) {
        const uint16_t *s = (const uint16_t *)stack + (size_t)j.first * fsz + (size_t)y0 * j.in_w + x0;
        unsigned short r[N];
#pragma unroll
        for (int u = 0; u < N; u++) r[u] = (t + u < tmax) ? __ldg(&s[(size_t)(t + u) * fsz]) : (unsigned short)0;
#pragma unroll
        for (int u = 0; u < N; u++) v[u] = (t + u < tmax) ? (float)((int)r[u] - bg) : 0.f;
    } else {
#pragma unroll
        for (int u = 0; u < N; u++) v[u] = (t + u < tmax) ? window_value(j, stack, x0, y0, t + u, bg) : 0.f;
    }
}

__host__ __device__ __forceinline__ void trace_origin(const Job &j, int trace, int &x0, int &y0)
{
    int pix = trace < j.npix ? trace : trace - j.npix;
    int ox = pix % j.out_w, oy = pix / j.out_w;
    x0 = (j.map_x0 + ox) * j.pixbinx;
    y0 = (j.map_y0 + oy) * j.pixbiny;
    if (trace >= j.npix) { x0 += j.cfx; y0 += j.cfy; }
}

// ---------------------------------------------------------------------------
// Bleach correction of one frame value (java:9682-9769):
//   v' = v / sqrt(f/f0) + f0 * (1 - sqrt(f/f0)),   t = frametime * (x + 0.5)
// with x the 1-based frame number.  Parameters per trace (kBleachStride floats):
//   polynomial: [0..8] coefficients in the Legendre basis of u(t), [13] u
//     scale, [14] u offset;
//   exponential: [0..4] the fit in the reference's form A, tau, C (single) or
//     A1, tau1, A2, tau2, C (double); the curve is evaluated as
//     f(t) = [13] + sum_c term_c(t) with rate k_c = [5], [6] (1/s) and
//     amplitude a_c = [7], [8]: term_c = a_c exp(-k_c t) when bit c of [14]
//     is clear, else -a_c t phi(k_c t), phi(x) = (1 - e^-x)/x as a series
//     (slow components, k_c t <= 0.5, where A and C of the reference's form
//     cancel);
//   all modes: [9] f0; [10] 1/f0; [11] valid flag; [12] centre c.
// ---------------------------------------------------------------------------
// t phi(k t) = (1 - e^{-kt}) / k for x = k t in [0, 0.5]: series to x^7
// (truncation below x^8 / 9! = 1.1e-8).
__device__ __forceinline__ float slow_exp_term(float k, float t)
{
    float x = k * t;
    float ph = fmaf(x, -1.f / 40320.f, 1.f / 5040.f);
    ph = fmaf(x, ph, -1.f / 720.f);
    ph = fmaf(x, ph, 1.f / 120.f);
    ph = fmaf(x, ph, -1.f / 24.f);
    ph = fmaf(x, ph, 1.f / 6.f);
    ph = fmaf(x, ph, -0.5f);
    ph = fmaf(x, ph, 1.f);
    return t * ph;
}

__device__ __forceinline__ float exp_component(const float *bp, int c, float t)
{
    const int flags = (int)bp[14];
    const float k = bp[5 + c], a = bp[7 + c];
    return ((flags >> c) & 1) ? -a * slow_exp_term(k, t) : a * __expf(-k * t);
}

__device__ __forceinline__ float bleach_f(const float *bp, int mode, int order, float t,
                                          const float *basis /* order+1 values at t */)
{
    if (mode == IMFCS_BLEACH_POLYNOMIAL) {
        float f = 0.f;
        for (int i = 0; i <= order; i++) f = fmaf(bp[i], basis[i], f);
        return f;
    } else if (mode == IMFCS_BLEACH_SINGLE_EXP) {
        return bp[13] + exp_component(bp, 0, t);
    } else {
        return bp[13] + exp_component(bp, 0, t) + exp_component(bp, 1, t);
    }
}

// v / sqrt(f/f0) + f0 (1 - sqrt(f/f0)) with one reciprocal square root,
// written as (v - f) / sqrt(f/f0) + f0 (f0 sqrt(f/f0) = f / sqrt(f/f0)):
// one subtraction, one FMA, and no 1 - sqrt(f/f0) cancellation when the
// curve is near f0.
__device__ __forceinline__ float bleach_correct(float v, float f, float f0, float inv_f0)
{
    return fmaf(v - f, rsqrtf(f * inv_f0), f0);
}

// Time of frame t (0-based) in the correction: frametime * (x + 0.5) with the
// 1-based frame number x = t + 1 (java:9747).
__device__ __forceinline__ float frame_time(const Job &j, int t) { return j.frametime * ((float)t + 1.5f); }

// Legendre polynomials P_0..P_order at u.
__device__ __forceinline__ void legendre(float u, int order, float *out)
{
    out[0] = 1.f;
    if (order >= 1) out[1] = u;
    for (int n = 1; n < order; n++)
        out[n + 1] = ((2 * n + 1) * u * out[n] - n * out[n - 1]) / (n + 1);
}

// ---------------------------------------------------------------------------
// FCS_3p model in FP32, internal units (um, s, um^2/s, um/s): value and
// gradient w.r.t. the 11 parameters (java:13131-13408).  The lateral term
// uses expm1 so that 1 - exp(-u^2) keeps full precision at long lag times.
// ---------------------------------------------------------------------------
struct ModelConst {
    float ax, ay, s, sz, rx, ry, inv_norm, q2, q3;   // inv_norm = fitobsvol / (4 (ax ay)^2)
};

__device__ __forceinline__ void lateral_1d_f(float a, float r, float v, float tau, float p0,
                                             float inv_p0, float &L, float &dL_dp0, float &dL_dv)
{
    const float inv_sqrtpi = 0.5641895835477563f;
    if (r == 0.f && v == 0.f) {   // autocorrelation without flow: the three terms collapse to two
        const float u = a * inv_p0;
        const float m = expm1f(-u * u), er = erff(u);
        L = 2.f * (p0 * inv_sqrtpi * m + a * er);
        dL_dp0 = 2.f * m * inv_sqrtpi;
        dL_dv = 0.f;   // (er2 + 2 er3 - er1) tau with er1 = er2, er3 = 0
        return;
    }
    float p1 = a + r - v * tau, p2 = a - r + v * tau, p3 = r - v * tau;
    float u1 = p1 * inv_p0, u2 = p2 * inv_p0, u3 = p3 * inv_p0;
    float m1 = expm1f(-u1 * u1), m2 = expm1f(-u2 * u2), m3 = expm1f(-u3 * u3);
    float e = m1 + m2 - 2.f * m3;   // e1 + e2 - 2 e3 exactly rewritten
    float er1 = erff(u1), er2 = erff(u2), er3 = erff(u3);
    L = p0 * inv_sqrtpi * e + p1 * er1 + p2 * er2 - 2.f * p3 * er3;
    dL_dp0 = e * inv_sqrtpi;
    dL_dv = (er2 + 2.f * er3 - er1) * tau;
}

struct CompTerms {
    float a, da_dd, da_dvx, da_dvy;
};

__device__ __forceinline__ void component_f(float d, float vx, float vy, const ModelConst &c,
                                            float tau, CompTerms &o)
{
    float p0 = sqrtf(fmaf(4.f * d, tau, c.s * c.s));
    float inv_p0 = 1.f / p0;
    float Lx, Ly, dLx0, dLy0, dLxv, dLyv;
    lateral_1d_f(c.ax, c.rx, vx, tau, p0, inv_p0, Lx, dLx0, dLxv);
    if (c.ay == c.ax && c.ry == c.rx && vy == vx) {   // square window, same offset and flow: same term
        Ly = Lx; dLy0 = dLx0; dLyv = dLxv;
    } else {
        lateral_1d_f(c.ay, c.ry, vy, tau, p0, inv_p0, Ly, dLy0, dLyv);
    }
    float dp0 = 2.f * tau * inv_p0;
    float lat = Lx * Ly * c.inv_norm;
    float dlat_dd = (dLx0 * Ly + Lx * dLy0) * dp0 * c.inv_norm;
    float inv_sz2 = 1.f / (c.sz * c.sz);
    float psp = rsqrtf(fmaf(4.f * d * tau, inv_sz2, 1.f));
    float dpsp = -2.f * tau * inv_sz2 * psp * psp * psp;
    o.a = lat * psp;
    o.da_dd = dlat_dd * psp + lat * dpsp;
    o.da_dvx = dLxv * Ly * c.inv_norm * psp;
    o.da_dvy = Lx * dLyv * c.inv_norm * psp;
}

// par: 11 parameters in internal units.  grad may be nullptr.
__device__ __forceinline__ float fcs_model_f(const float *par, const ModelConst &c, float tau,
                                             float *grad, bool comp2, bool comp3)
{
    float N = par[0], F2 = par[5], F3 = par[7], Ft = par[9], Tt = par[10];
    CompTerms c1, c2 = {0, 0, 0, 0}, c3 = {0, 0, 0, 0};
    component_f(par[1], par[2], par[3], c, tau, c1);
    if (comp2) component_f(par[6], par[2], par[3], c, tau, c2);
    if (comp3) component_f(par[8], par[2], par[3], c, tau, c3);
    float et = (Tt != 0.f) ? __expf(-tau / Tt) : 0.f;
    float trip = 1.f + Ft / (1.f - Ft) * et;
    float Z = 1.f - F2 - F3 + c.q2 * F2 + c.q3 * F3;
    float w1 = 1.f - F2 - F3, w2 = c.q2 * c.q2 * F2, w3 = c.q3 * c.q3 * F3;
    float S = w1 * c1.a + w2 * c2.a + w3 * c3.a;
    float iZ = 1.f / Z, iN = 1.f / N;
    float base = S * iZ * iZ;
    float val = base * iN * trip + par[4];
    if (grad) {
        float k = trip * iN * iZ * iZ;
        grad[0] = -base * trip * iN * iN;
        grad[1] = k * w1 * c1.da_dd;
        grad[2] = k * (w1 * c1.da_dvx + w2 * c2.da_dvx + w3 * c3.da_dvx);
        grad[3] = k * (w1 * c1.da_dvy + w2 * c2.da_dvy + w3 * c3.da_dvy);
        grad[4] = 1.f;
        grad[5] = trip * iN * ((c.q2 * c.q2 * c2.a - c1.a) * iZ * iZ - 2.f * S * (c.q2 - 1.f) * iZ * iZ * iZ);
        grad[6] = k * w2 * c2.da_dd;
        grad[7] = trip * iN * ((c.q3 * c.q3 * c3.a - c1.a) * iZ * iZ - 2.f * S * (c.q3 - 1.f) * iZ * iZ * iZ);
        grad[8] = k * w3 * c3.da_dd;
        float omf = 1.f - Ft;
        grad[9] = base * iN * et / (omf * omf);
        grad[10] = (Tt != 0.f) ? base * iN * Ft / omf * et * tau / (Tt * Tt) : 0.f;
    }
    return val;
}

// FP64 value of the same model (no gradient), used for the residuals of the
// final Gauss-Newton polish so that the located minimum does not carry the
// FP32 evaluation error (~5e-7 relative) of fcs_model_f.
struct ModelConstD {
    double ax, ay, s, sz, rx, ry, inv_norm, q2, q3;
};

__device__ __forceinline__ double lateral_1d_d(double a, double r, double v, double tau, double p0)
{
    const double inv_sqrtpi = 0.56418958354775628695;
    if (r == 0.0 && v == 0.0) {   // autocorrelation without flow: the three terms collapse to two
        const double u = a / p0;
        return 2.0 * (p0 * inv_sqrtpi * expm1(-u * u) + a * erf(u));
    }
    double p1 = a + r - v * tau, p2 = a - r + v * tau, p3 = r - v * tau;
    double u1 = p1 / p0, u2 = p2 / p0, u3 = p3 / p0;
    double e = expm1(-u1 * u1) + expm1(-u2 * u2) - 2.0 * expm1(-u3 * u3);
    return p0 * inv_sqrtpi * e + p1 * erf(u1) + p2 * erf(u2) - 2.0 * p3 * erf(u3);
}

__device__ __forceinline__ double component_d(double d, double vx, double vy, const ModelConstD &c, double tau)
{
    double p0 = sqrt(4.0 * d * tau + c.s * c.s);
    const double lx = lateral_1d_d(c.ax, c.rx, vx, tau, p0);
    const double ly = (c.ay == c.ax && c.ry == c.rx && vy == vx) ? lx : lateral_1d_d(c.ay, c.ry, vy, tau, p0);
    double lat = lx * ly * c.inv_norm;
    return lat / sqrt(1.0 + 4.0 * d * tau / (c.sz * c.sz));
}

__device__ __forceinline__ double fcs_model_value_d(const double *par, const ModelConstD &c, double tau,
                                                    bool comp2, bool comp3)
{
    double N = par[0], F2 = par[5], F3 = par[7], Ft = par[9], Tt = par[10];
    double a1 = component_d(par[1], par[2], par[3], c, tau);
    double a2 = comp2 ? component_d(par[6], par[2], par[3], c, tau) : 0.0;
    double a3 = comp3 ? component_d(par[8], par[2], par[3], c, tau) : 0.0;
    double et = (Tt != 0.0) ? exp(-tau / Tt) : 0.0;
    double trip = 1.0 + Ft / (1.0 - Ft) * et;
    double Z = 1.0 - F2 - F3 + c.q2 * F2 + c.q3 * F3;
    double S = (1.0 - F2 - F3) * a1 + c.q2 * c.q2 * F2 * a2 + c.q3 * c.q3 * F3 * a3;
    return S / (Z * Z) / N * trip + par[4];
}

// Unit of each parameter in the internal system (multiply internal by unit
// to get SI): N, D[um^2/s], vx, vy [um/s], G, F2, D2, F3, D3, Ftrip, Ttrip [s].
__host__ __device__ __forceinline__ double param_unit(int i)
{
    switch (i) {
    case 1: case 6: case 8: return 1e-12;
    case 2: case 3: return 1e-6;
    default: return 1.0;
    }
}

// ---------------------------------------------------------------------------
// Warp helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float warp_sum(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace imfcs
