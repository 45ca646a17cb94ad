// imfcs_lm_tirf.cu -- the LM fit of the plugin's default model, specialised:
// FCS_3p (java:13131-13408) with one component, no flow, no triplet, N, D and
// G free (the other parameters held at zero), up to kMaxPts points,
// step-mode stopping rule.  Same algorithm, stopping rules and FP32
// operation order as lm_kernel (imfcs_lm.cuh): phase 1 LM on FP32 model
// values, Newton finish with a forward-difference Hessian, FP32 then FP64
// residuals.  The model is evaluated from three scalars instead of the
// 11-parameter vector, so the parameters live in registers (no local-memory
// arrays indexed at run time) and the executed code is a few kilobytes --
// the generic kernel stalls on instruction fetch and local-memory loads.
//
// Two compile-time variants widen it to the rest of the plugin's fits of
// this model: OFF, the spatial cross-correlation model (window offsets rx,
// ry: the three-term lateral factor), and GLS, the fit on the data and model
// whitened by L^-1 of the regularised covariance (GLSFit, java:10622-10789).
// With GLS the model enters through u = L^-1 a and v = L^-1 da/dD of its
// N-free part a: L^-1 f = u / N + G L^-1 1, so each evaluation is two
// triangular products per warp (L^-1 in shared memory), and the FP64
// residuals transform the FP64 values of a.
#include "imfcs_ff.cuh"
#include "imfcs_lm.cuh"

namespace imfcs {

struct TirfC {
    float ax, ay, rx, ry, s2, inv_sz2, inv_norm;
    double axd, ayd, rxd, ryd, sd, inv_sz2d, inv_normd;
    f2 s2f, inv_normf;   // float-float copies for the precise residuals
    bool square;         // ax == ay (and rx == ry): the two lateral factors coincide
    bool axial;          // the axial factor can differ from 1 in FP64 (finite sz)
};

// Lateral factor of a square-pixel window without offset or flow (the
// two-term form of lateral_1d_f).
__device__ __forceinline__ void tirf_lat(float a, float p0, float inv_p0, float &L, float &dL)
{
    const float inv_sqrtpi = 0.5641895835477563f;
    const float u = a * inv_p0;
    const float m = expm1f(-u * u), er = erff(u);
    L = 2.f * (p0 * inv_sqrtpi * m + a * er);
    dL = 2.f * m * inv_sqrtpi;
}

// The N-free part of the model a(D, tau) = lateral x axial factor and
// da/dD in FP32, internal units (the model is a / N + G).
template <bool OFF>
__device__ __noinline__ void tirf_terms(float D, const TirfC &c, float tau, float &a, float &da)
{
    const float p0 = sqrtf(fmaf(4.f * D, tau, c.s2));
    const float inv_p0 = 1.f / p0;
    float Lx, dLx, Ly, dLy;
    if (OFF) {
        float dv;
        lateral_1d_f(c.ax, c.rx, 0.f, tau, p0, inv_p0, Lx, dLx, dv);
        if (c.square) { Ly = Lx; dLy = dLx; }
        else lateral_1d_f(c.ay, c.ry, 0.f, tau, p0, inv_p0, Ly, dLy, dv);
    } else {
        tirf_lat(c.ax, p0, inv_p0, Lx, dLx);
        if (c.square) { Ly = Lx; dLy = dLx; }
        else tirf_lat(c.ay, p0, inv_p0, Ly, dLy);
    }
    const float dp0 = 2.f * tau * inv_p0;
    const float lat = Lx * Ly * c.inv_norm;
    const float dlat = (dLx * Ly + Lx * dLy) * dp0 * c.inv_norm;
    const float psp = rsqrtf(fmaf(4.f * D * tau, c.inv_sz2, 1.f));
    const float dpsp = -2.f * tau * c.inv_sz2 * psp * psp * psp;
    a = lat * psp;
    da = dlat * psp + lat * dpsp;
}

// Model value and gradient (d/dN, d/dD; d/dG = 1) in FP32, internal units;
// mag = |a/N| + |G|, the magnitude of the summed terms (the rounding error
// of the value is relative to it).
template <bool OFF>
__device__ __forceinline__ float tirf_f(float N, float D, float G, const TirfC &c, float tau, float &gN, float &gD,
                                        float &mag)
{
    float a, da;
    tirf_terms<OFF>(D, c, tau, a, da);
    const float iN = 1.f / N;
    gN = -a * iN * iN;
    gD = iN * da;
    const float aN = __fmul_rn(a, iN);
    mag = fabsf(aN) + fabsf(G);
    return aN + G;
}

// FP64 N-free model part a (the precise residuals: a / N + G), with as few
// FP64 divisions and square roots as the accuracy allows (GB300 issues FP64
// at 1/64 of the FP32 rate): 1/p0 from one reciprocal square root, and the
// axial factor (1 + 4 D tau / sz^2)^(-1/2) only where it differs from 1 in
// FP64 (a TIRF model's sz is ~1e6 um: 4 D tau / sz^2 < 1e-17 and the factor
// rounds to exactly 1).  The offset lateral factor (OFF) divides by p0.
template <bool OFF>
__device__ __noinline__ double tirf_a_d(double D, const TirfC &c, double tau)
{
    const double inv_sqrtpi = 0.56418958354775628695;
    const double p2 = 4.0 * D * tau + c.sd * c.sd;
    const double ip0 = rsqrt(p2);
    const double p0 = p2 * ip0;
    double lx, ly;
    if (OFF) {
        lx = lateral_1d_d(c.axd, c.rxd, 0.0, tau, p0);
        ly = c.square ? lx : lateral_1d_d(c.ayd, c.ryd, 0.0, tau, p0);
    } else {
        double u = c.axd * ip0;
        lx = 2.0 * (p0 * inv_sqrtpi * expm1(-u * u) + c.axd * erf(u));
        ly = lx;
        if (!c.square) {
            u = c.ayd * ip0;
            ly = 2.0 * (p0 * inv_sqrtpi * expm1(-u * u) + c.ayd * erf(u));
        }
    }
    double a1 = lx * ly * c.inv_normd;
    const double ax = 4.0 * D * tau * c.inv_sz2d;
    if (ax > 1e-17) a1 *= rsqrt(1.0 + ax);
    return a1;
}

// Float-float model value for the precise residuals: about 1e-12 relative,
// far below what the residuals need (the data are FP32), on the FP32 pipes.
// erf(u) = u sum_n e_n x^n with e_n = (2/sqrt(pi)) (-1)^n / (n! (2n+1)) and
// expm1(-x) = -x sum_n q_n x^n with q_n = (-1)^n / (n+1)!, x = u^2, are the
// Taylor series, truncated at n = 15: for u <= 1 the first omitted terms are
// below 3e-14 and 5e-14.  Points with u > 1 (windows much wider than the
// PSF) or an axial factor different from 1 in FP64 (SPIM) take the FP64
// model instead.
constexpr int kSeriesN = 16;

// The series coefficients as float-float (hi = the float nearest the FP64
// value, lo = the float nearest the remainder), evaluated at compile time.
struct SeriesTab {
    float eh[kSeriesN], el[kSeriesN], qh[kSeriesN], ql[kSeriesN];
};
constexpr SeriesTab make_series_tab()
{
    SeriesTab t{};
    const double two_sqrtpi = 1.1283791670955125739;   // 2 / sqrt(pi)
    double fact = 1.0;                                 // n!
    for (int n = 0; n < kSeriesN; n++) {
        if (n > 0) fact *= n;
        const double en = ((n & 1) ? -1.0 : 1.0) * two_sqrtpi / (fact * (2 * n + 1));
        const double qn = ((n & 1) ? -1.0 : 1.0) / (fact * (n + 1));
        t.eh[n] = (float)en;
        t.el[n] = (float)(en - (double)t.eh[n]);
        t.qh[n] = (float)qn;
        t.ql[n] = (float)(qn - (double)t.qh[n]);
    }
    return t;
}
__constant__ SeriesTab kSeries = make_series_tab();

__device__ __forceinline__ f2 ff_const(const float *hi, const float *lo, int n) { return {hi[n], lo[n]}; }

// L = 2 (p0 / sqrt(pi) expm1(-u^2) + a erf(u)), u = a / p0 (float-float);
// false when u > 1
__device__ __forceinline__ bool tirf_lat_ff(float a, f2 p0, f2 ip0, f2 &L)
{
    const f2 u = f2_mul_f(ip0, a);
    if (!(u.hi <= 1.f)) return false;
    const f2 x = f2_mul(u, u);
    f2 pe = ff_const(kSeries.eh, kSeries.el, kSeriesN - 1), pq = ff_const(kSeries.qh, kSeries.ql, kSeriesN - 1);
#pragma unroll
    for (int n = kSeriesN - 2; n >= 0; n--) {
        pe = f2_add(f2_mul(pe, x), ff_const(kSeries.eh, kSeries.el, n));
        pq = f2_add(f2_mul(pq, x), ff_const(kSeries.qh, kSeries.ql, n));
    }
    const f2 er = f2_mul(u, pe);                     // erf(u)
    const f2 m = f2_neg(f2_mul(x, pq));               // expm1(-u^2)
    const f2 inv_sqrtpi = {5.641896129e-01f, -2.931769139e-08f};   // 1/sqrt(pi) as float-float
    const f2 t1 = f2_mul(f2_mul(p0, inv_sqrtpi), m);
    const f2 t2 = f2_mul_f(er, a);
    const f2 sum = f2_add(t1, t2);
    L = {2.f * sum.hi, 2.f * sum.lo};
    return true;
}

// N-free model part a in float-float at D; false where the FP64 model is
// needed (see above).
__device__ __forceinline__ bool tirf_a_ff(f2 D, const TirfC &c, float tau, f2 &lat)
{
    if (c.axial) return false;
    // p0^2 = 4 D tau + s^2 (4 tau exact), 1/p0 by one Newton step on
    // rsqrtf: e = 1 - p2 r^2, 1/p0 = r + r e / 2 (error ~e^2)
    const f2 p2 = f2_add(f2_mul_f(D, 4.f * tau), c.s2f);
    const float r = rsqrtf(p2.hi);
    const f2 pr2 = f2_mul_f(f2_mul_f(p2, r), r);
    const float e = (1.f - pr2.hi) - pr2.lo;
    const f2 ip0 = f2_two_sum(r, 0.5f * r * e);
    const f2 p0 = f2_mul(p2, ip0);
    f2 Lx, Ly;
    if (!tirf_lat_ff(c.ax, p0, ip0, Lx)) return false;
    if (c.square) Ly = Lx;
    else if (!tirf_lat_ff(c.ay, p0, ip0, Ly)) return false;
    lat = f2_mul(f2_mul(Lx, Ly), c.inv_normf);
    return true;
}

struct Tirf3 {
    float A[9];
    float g[3];
    float chi2;      // FP32 phases
    double chi2d;    // FP64-residual evaluations
    float fmag;      // sum w (|a/N| + |G|)^2: scale of the model values (FP32 phases)
};

// Per-warp shared memory of a GLS fit: L^-1 (packed lower, float), its row
// sums (L^-1 1, float and FP64), and the staged N-free model part a, da/dD
// (FP32) and a (FP64) of the points.
struct GlsSh {
    float *L, *l1, *sa, *sda;
    double *sfd, *l1d;
};

__device__ __forceinline__ void tirf_reduce(float (&acc)[9], Tirf3 &s)
{
    int q = 0;
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int t = 0; t <= p; t++) {
            const float v = warp_sum(acc[q++]);
            s.A[p * 3 + t] = v;
            s.A[t * 3 + p] = v;
        }
#pragma unroll
    for (int p = 0; p < 3; p++) s.g[p] = warp_sum(acc[q++]);
}

__device__ __forceinline__ void tirf_accumulate(float (&acc)[9], const float (&gr)[3], float w, float r)
{
    int q = 0;
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int t = 0; t <= p; t++) acc[q++] += w * gr[p] * gr[t];
#pragma unroll
    for (int p = 0; p < 3; p++) acc[q++] += w * gr[p] * r;
}

// GLS: stage a, da/dD of the warp's points (and, for the precise residuals,
// a in FP64) in shared memory.
template <bool OFF>
__device__ __forceinline__ void gls_stage(const TirfC &c, float D, double Dd, const float *xl, int n, int lane,
                                          const GlsSh &g, bool precise)
{
#pragma unroll
    for (int m = 0; m < kPtsPerLane; m++) {
        const int i = lane + 32 * m;
        if (i < n) {
            float a, da;
            tirf_terms<OFF>(D, c, xl[m], a, da);
            g.sa[i] = a;
            g.sda[i] = da;
            if (precise) {
                f2 lat;
                g.sfd[i] = (!OFF && tirf_a_ff(f2_from_d(Dd), c, xl[m], lat)) ? (double)lat.hi + (double)lat.lo
                                                                           : tirf_a_d<OFF>(Dd, c, (double)xl[m]);
            }
        }
    }
    __syncwarp();
}

// GLS row r of the whitened model: u = (L^-1 a)_r, v = (L^-1 da/dD)_r.
__device__ __forceinline__ void gls_row(const GlsSh &g, int r, float &u, float &v)
{
    const float *Lr = g.L + r * (r + 1) / 2;
    u = 0.f;
    v = 0.f;
    for (int k = 0; k <= r; k++) {
        const float l = Lr[k];
        u = fmaf(l, g.sa[k], u);
        v = fmaf(l, g.sda[k], v);
    }
}

// One evaluation over the fit's points (warp): chi^2, J^T W J, J^T W r with
// FP32 residuals.  No FP64 operation: GB300 issues FP64 at 1/64 of the FP32
// rate, and the FP32 phases evaluate the model some twenty times per fit.
template <bool OFF, bool GLS>
__device__ __noinline__ void tirf_eval32(const TirfC &c, float N, float D, float G, const float *yl,
                                         const float *wl, const float *xl, int n, int lane, Tirf3 &s,
                                         const GlsSh &g)
{
    float acc[9];
#pragma unroll
    for (int i = 0; i < 9; i++) acc[i] = 0.f;
    float c2f = 0.f, fm = 0.f;
    if (GLS) {
        gls_stage<OFF>(c, D, 0.0, xl, n, lane, g, false);
        const float iN = 1.f / N;
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            const int r = lane + 32 * m;
            if (r < n) {
                float u, v;
                gls_row(g, r, u, v);
                const float gr[3] = {-u * iN * iN, iN * v, g.l1[r]};
                const float f = __fmul_rn(u, iN) + G * g.l1[r];
                const float res = yl[m] - f;
                c2f = fmaf(res, res, c2f);
                tirf_accumulate(acc, gr, 1.f, res);
            }
        }
        __syncwarp();
    } else {
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            const int i = lane + 32 * m;
            if (i < n) {
                float gr[3], mag;
                gr[2] = 1.f;
                const float f = tirf_f<OFF>(N, D, G, c, xl[m], gr[0], gr[1], mag);
                const float w = wl[m];
                const float r = yl[m] - f;
                c2f = fmaf(w * r, r, c2f);
                fm = fmaf(w * mag, mag, fm);
                tirf_accumulate(acc, gr, w, r);
            }
        }
    }
    tirf_reduce(acc, s);
    s.chi2 = warp_sum(c2f);
    s.chi2d = 0.0;
    s.fmag = warp_sum(fm);
}

// The same with residuals of the model value in float-float at the FP64
// parameters (Nd, Dd, Gd) -- FP64 model where the series do not apply --
// the Jacobian in FP32 at their FP32 copies; chi^2 reduced in float-float.
// GLS: residuals of the FP64 whitened model (L^-1 applied in FP64 to the
// FP64 values of a), chi^2 in FP64.
template <bool OFF, bool GLS>
__device__ __noinline__ void tirf_eval64(const TirfC &c, double Nd, double Dd, double Gd, const float *yl,
                                         const float *wl, const float *xl, int n, int lane, Tirf3 &s,
                                         const GlsSh &g)
{
    const float N = (float)Nd, D = (float)Dd, G = (float)Gd;
    const double inv_Nd = 1.0 / Nd;
    float acc[9];
#pragma unroll
    for (int i = 0; i < 9; i++) acc[i] = 0.f;
    if (GLS) {
        gls_stage<OFF>(c, D, Dd, xl, n, lane, g, true);
        const float iN = 1.f / N;
        double c2 = 0.0;
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            const int r = lane + 32 * m;
            if (r < n) {
                float u, v;
                gls_row(g, r, u, v);
                const float gr[3] = {-u * iN * iN, iN * v, g.l1[r]};
                const float *Lr = g.L + r * (r + 1) / 2;
                double U = 0.0;
                for (int k = 0; k <= r; k++) U = fma((double)Lr[k], g.sfd[k], U);
                const double rr = (double)yl[m] - fma(U, inv_Nd, Gd * g.l1d[r]);
                c2 = fma(rr, rr, c2);
                tirf_accumulate(acc, gr, 1.f, (float)rr);
            }
        }
        __syncwarp();
        tirf_reduce(acc, s);
        s.chi2d = warp_sum_d(c2);
        s.chi2 = (float)s.chi2d;
        s.fmag = 0.f;
        return;
    }
    const f2 inv_Nf = f2_from_d(inv_Nd), Df = f2_from_d(Dd), Gf = f2_from_d(Gd);
    f2 c2acc = {0.f, 0.f};
#pragma unroll
    for (int m = 0; m < kPtsPerLane; m++) {
        const int i = lane + 32 * m;
        if (i < n) {
            float gr[3], mag;
            gr[2] = 1.f;
            tirf_f<OFF>(N, D, G, c, xl[m], gr[0], gr[1], mag);
            const float w = wl[m];
            f2 fv, lat;
            if (!OFF && tirf_a_ff(Df, c, xl[m], lat)) fv = f2_add(f2_mul(lat, inv_Nf), Gf);
            else fv = f2_from_d(fma(tirf_a_d<OFF>(Dd, c, (double)xl[m]), inv_Nd, Gd));
            const f2 rr = f2_add(f2_from_f(yl[m]), f2_neg(fv));
            const float r = f2_val(rr);
            c2acc = f2_add(c2acc, f2_mul_f(f2_mul(rr, rr), w));
            tirf_accumulate(acc, gr, w, r);
        }
    }
    tirf_reduce(acc, s);
    for (int o = 16; o > 0; o >>= 1) {
        const f2 other = {__shfl_xor_sync(0xffffffffu, c2acc.hi, o), __shfl_xor_sync(0xffffffffu, c2acc.lo, o)};
        c2acc = f2_add(c2acc, other);
    }
    s.chi2d = (double)c2acc.hi + (double)c2acc.lo;
    s.chi2 = c2acc.hi + c2acc.lo;
    s.fmag = 0.f;
}

// dispatch by phase
template <bool OFF, bool GLS>
__device__ __forceinline__ void tirf_eval(const TirfC &c, float N, float D, float G, double Nd, double Dd, double Gd,
                                          const float *yl, const float *wl, const float *xl, int n, int lane,
                                          bool precise, Tirf3 &s, const GlsSh &g)
{
    if (precise) tirf_eval64<OFF, GLS>(c, Nd, Dd, Gd, yl, wl, xl, n, lane, s, g);
    else tirf_eval32<OFF, GLS>(c, N, D, G, yl, wl, xl, n, lane, s, g);
}

__device__ __forceinline__ float tirf_sig(const Tirf3 &s, int i) { return rsqrtf(fmaxf(s.A[i * 3 + i], 1e-30f)); }

// Floats of shared memory per warp of a GLS fit with n points: L^-1, l1, a,
// da/dD, then (8-byte aligned) a in FP64 and l1 in FP64.
__host__ __device__ __forceinline__ int gls_warp_floats(int n)
{
    return ((n * (n + 1) / 2 + 3 * n + 1) & ~1) + 4 * n;
}

// Bound on the relative rounding error of the FP32 model value (erff and
// expm1f within a few ulp, ~15 roundings of the lateral, axial and final
// terms): 4e-6, some 70 ulp.
constexpr float kModelRound = 4e-6f;

template <bool OFF, bool GLS>
__global__ void __launch_bounds__(128) lm_tirf_kernel(FitArgs a)
{
    extern __shared__ float tsh[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int n = a.npts;
    const int gw = blockIdx.x * wpb + wib, nw = gridDim.x * wpb;
    TirfC c;
    c.ax = a.mc.ax; c.ay = a.mc.ay; c.rx = a.mc.rx; c.ry = a.mc.ry;
    c.s2 = a.mc.s * a.mc.s; c.inv_sz2 = 1.f / (a.mc.sz * a.mc.sz);
    c.inv_norm = a.mc.inv_norm;
    c.axd = a.mc.ax; c.ayd = a.mc.ay; c.rxd = a.mc.rx; c.ryd = a.mc.ry;
    c.sd = a.mc.s; c.inv_normd = a.mc.inv_norm;
    c.inv_sz2d = 1.0 / ((double)a.mc.sz * (double)a.mc.sz);
    c.square = a.mc.ay == a.mc.ax && a.mc.ry == a.mc.rx;
    c.s2f = f2_two_prod(a.mc.s, a.mc.s);
    c.inv_normf = f2_from_f(a.mc.inv_norm);
    // 4 D tau / sz^2 at the largest D and lag time a fit can reach is far
    // below FP64 resolution for a TIRF sz; the axial factor is then exactly 1
    c.axial = !(c.inv_sz2d * 4e6 < 1e-17);
    float xl[kPtsPerLane];
#pragma unroll
    for (int m = 0; m < kPtsPerLane; m++) {
        const int i = lane + 32 * m;
        xl[m] = i < n ? __ldg(&a.x[i]) : 0.f;
    }
    GlsSh g = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const int npairs = n * (n + 1) / 2;
    if (GLS) {
        float *base = tsh + (size_t)wib * gls_warp_floats(n);
        g.L = base;
        g.l1 = base + npairs;
        g.sa = g.l1 + n;
        g.sda = g.sa + n;
        g.sfd = (double *)(base + ((npairs + 3 * n + 1) & ~1));
        g.l1d = g.sfd + n;
    }
    for (int fit = a.counter ? lm_next_fit(a, 0, 0, lane) : gw; fit < a.nfits; fit = lm_next_fit(a, fit, nw, lane)) {
        if (a.todo && !__ldg(&a.todo[fit])) continue;
        if (GLS) {
            // this fit's L^-1 and its row sums (the whitened constant G)
            const float *src = a.linv + (size_t)fit * npairs;
            for (int i = lane; i < npairs; i += 32) g.L[i] = __ldg(&src[i]);
            __syncwarp();
            for (int r = lane; r < n; r += 32) {
                const float *Lr = g.L + r * (r + 1) / 2;
                float s1 = 0.f;
                double s1d = 0.0;
                for (int k = 0; k <= r; k++) { s1 += Lr[k]; s1d += (double)Lr[k]; }
                g.l1[r] = s1;
                g.l1d[r] = s1d;
            }
            __syncwarp();
        }
        float yl[kPtsPerLane], wl[kPtsPerLane];
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            const int i = lane + 32 * m;
            yl[m] = i < n ? __ldg(&a.y[(size_t)fit * n + i]) : 0.f;
            wl[m] = i < n ? (a.w ? __ldg(&a.w[(size_t)fit * n + i]) : 1.f) : 0.f;
        }
        const float *ip = a.init + (size_t)fit * a.init_stride;
        // free parameters N, D, G (vector indices 0, 1, 4): FP32 in the FP32
        // phases, FP64 from the FP64-residual Newton steps on
        float pf[3] = {__ldg(&ip[0]), __ldg(&ip[1]), __ldg(&ip[4])};
        double pd[3] = {0.0, 0.0, 0.0};
        bool precise = false;     // parameters and chi^2 held in FP64 (pd, chi2d)
        bool retried = false;     // Newton left its region once: FP32 LM to 1e-4 sigma, then Newton again
        Tirf3 s;
        tirf_eval<OFF, GLS>(c, pf[0], pf[1], pf[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, s, g);
        int state = IMFCS_STATE_MAX_ITERATIONS, it = 0, nprec = 0;
        float lambda = 1e-3f;
        if (!isfinite(s.chi2)) state = IMFCS_STATE_SINGULAR_HESSIAN;
        for (it = 0; state == IMFCS_STATE_MAX_ITERATIONS && it < a.max_iter; it++) {
            float h[3];
            bool to_precise = false;
            {
                float hg[3];
                if (solve_scaled<3>(s.A, s.g, 3, 0.f, hg)) {
                    bool conv = true;
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        const float sig = tirf_sig(s, i);
                        const float tol = precise ? 1e-7f * fabsf(pf[i]) + 1e-5f * sig : (retried ? 1e-4f : 1e-3f) * sig;
                        conv = conv && (fabsf(hg[i]) <= tol);
                    }
                    if (conv) {
                        if (precise) { state = IMFCS_STATE_CONVERGED; break; }
                        to_precise = true;
                    }
                }
            }
            if (!to_precise) {
                if (!solve_scaled<3>(s.A, s.g, 3, lambda, h)) {
                    lambda *= 10.f;
                    if (lambda > 1e15f) { state = IMFCS_STATE_SINGULAR_HESSIAN; break; }
                    continue;
                }
                Tirf3 sn;
                float pnf[3];
                double pnd[3] = {0.0, 0.0, 0.0};
                bool better;
                if (precise) {
#pragma unroll
                    for (int i = 0; i < 3; i++) { pnd[i] = pd[i] + (double)h[i]; pnf[i] = (float)pnd[i]; }
                    tirf_eval<OFF, GLS>(c, pnf[0], pnf[1], pnf[2], pnd[0], pnd[1], pnd[2], yl, wl, xl, n, lane, true, sn, g);
                    nprec++;
                    better = isfinite(sn.chi2d) && sn.chi2d < s.chi2d;
                } else {
#pragma unroll
                    for (int i = 0; i < 3; i++) pnf[i] = pf[i] + h[i];
                    tirf_eval<OFF, GLS>(c, pnf[0], pnf[1], pnf[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, sn, g);
                    better = isfinite(sn.chi2) && sn.chi2 < s.chi2;
                }
                if (better) {
#pragma unroll
                    for (int i = 0; i < 3; i++) { pd[i] = pnd[i]; pf[i] = pnf[i]; }
                    s = sn;
                    lambda = fmaxf(lambda * 0.1f, 1e-9f);
                } else {
                    lambda *= 10.f;
                    if (lambda > (precise ? 1e10f : 1e6f)) {
                        if (precise) { state = IMFCS_STATE_CONVERGED; it++; break; }
                        to_precise = true;
                    }
                }
                if (nprec > 60) { state = IMFCS_STATE_CONVERGED; it++; break; }
            }
            if (to_precise) {
                // Newton finish (see lm_kernel): forward-difference Hessian
                // of chi^2/2 from the FP32 gradient, FP32 steps to its
                // stationary point, then FP64-residual steps until the step
                // is below 1e-4 sigma + 1e-7 |p|.
                float H[9];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float eps = 0.1f * tirf_sig(s, i);
                    float pe[3] = {pf[0], pf[1], pf[2]};
                    pe[i] = pf[i] + eps;
                    const float de = pe[i] - pf[i];
                    Tirf3 se;
                    tirf_eval<OFF, GLS>(c, pe[0], pe[1], pe[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, se, g);
#pragma unroll
                    for (int r = 0; r < 3; r++) H[r * 3 + i] = (s.g[r] - se.g[r]) / de;
                }
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int q = 0; q < r; q++) {
                        const float v = 0.5f * (H[r * 3 + q] + H[q * 3 + r]);
                        H[r * 3 + q] = v;
                        H[q * 3 + r] = v;
                    }
                bool newton_done = false, left = false, stationary = false;
#pragma unroll 1
                for (int ni = 0; ni < 7 && !left; ni++) {
                    const bool fp64 = ni >= 3;
                    if (!OFF && !GLS && fp64 && !precise && stationary) {
                        // At the FP32 gradient's stationary point.  The FP32
                        // model value's rounding error (below kModelRound of
                        // the summed terms' magnitude, |a/N| + |G|) moves
                        // the minimum by at most B sigma_i in parameter i,
                        // B = kModelRound sqrt(sum w (|a/N| + |G|)^2)
                        // (Cauchy-Schwarz in the metric of J^T W J).  Where
                        // that is below 1e-5 of N and of D, the FP64 step
                        // cannot matter at the 1e-4 parity bar: skip it.
                        // (Not for the offset lateral factor, whose terms
                        // cancel, nor for the whitened model, whose values
                        // are sums over all points.)
                        const float B = kModelRound * sqrtf(s.fmag);
                        if (B * tirf_sig(s, 0) <= 1e-5f * fabsf(pf[0]) && B * tirf_sig(s, 1) <= 1e-5f * fabsf(pf[1])) {
                            newton_done = true;
                            break;
                        }
                    }
                    if (fp64) {
                        if (!precise) {
#pragma unroll
                            for (int i = 0; i < 3; i++) pd[i] = (double)pf[i];
                            precise = true;
                        }
                        tirf_eval<OFF, GLS>(c, pf[0], pf[1], pf[2], pd[0], pd[1], pd[2], yl, wl, xl, n, lane, true, s, g);
                        if (!isfinite(s.chi2d)) { left = true; break; }
                    }
                    float hn[3];
                    if (!solve_scaled<3>(H, s.g, 3, 0.f, hn)) { left = true; break; }
                    bool small = true;
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        const float sig = tirf_sig(s, i);
                        if (!(fabsf(hn[i]) <= 0.05f * sig)) left = true;
                        small = small && (fabsf(hn[i]) <= 1e-4f * sig + (fp64 ? 1e-7f * fabsf(pf[i]) : 0.f));
                    }
                    if (left) break;
                    if (fp64) {
#pragma unroll
                        for (int i = 0; i < 3; i++) { pd[i] += (double)hn[i]; pf[i] = (float)pd[i]; }
                        if (small) { newton_done = true; break; }
                    } else {
#pragma unroll
                        for (int i = 0; i < 3; i++) pf[i] += hn[i];
                        if (small) {
                            ni = 2;
                            stationary = true;
                        } else {
                            tirf_eval<OFF, GLS>(c, pf[0], pf[1], pf[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, s, g);
                        }
                    }
                }
                if (newton_done) { state = IMFCS_STATE_CONVERGED; it++; break; }
                if (!retried) {
                    // Newton left its quadratic region (a step above 0.05
                    // sigma) or met an indefinite Hessian: back to FP32 LM,
                    // to the tighter 1e-4 sigma, and Newton from there -- an
                    // LM on FP64-residual evaluations costs ~10x an FP32
                    // iteration and runs for tens of iterations, and the few
                    // fits that take it set the duration of the whole launch
                    retried = true;
                    if (precise) {
#pragma unroll
                        for (int i = 0; i < 3; i++) pf[i] = (float)pd[i];
                        precise = false;
                    }
                    tirf_eval<OFF, GLS>(c, pf[0], pf[1], pf[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, s, g);
                    lambda = 1e-3f;
                    continue;
                }
                // otherwise LM on the FP64-residual model
                if (!precise) {
#pragma unroll
                    for (int i = 0; i < 3; i++) pd[i] = (double)pf[i];
                    precise = true;
                }
                tirf_eval<OFF, GLS>(c, pf[0], pf[1], pf[2], pd[0], pd[1], pd[2], yl, wl, xl, n, lane, true, s, g);
                lambda = 1e-3f;
            }
        }
        if (lane == 0) {
            float *o = a.out_par + (size_t)fit * a.out_stride;
            for (int i = 0; i < a.np; i++) o[i] = __ldg(&ip[i]);
            o[0] = precise ? (float)pd[0] : pf[0];
            o[1] = precise ? (float)pd[1] : pf[1];
            o[4] = precise ? (float)pd[2] : pf[2];
            if (a.out_chi2) a.out_chi2[fit] = s.chi2;
            if (a.out_state) a.out_state[fit] = state;
            if (a.out_iter) a.out_iter[fit] = it;
            if (a.out_hess)
                for (int i = 0; i < 9; i++) a.out_hess[(size_t)fit * 9 + i] = s.A[i];
        }
        __syncwarp();
    }
}

// Whether a fit can take the specialised kernel: ACF model, step mode,
// shared constants (window offsets allowed: OFF), OLS or GLS, N, D, G free
// in that order and every other parameter held at zero (tirf_zero_held:
// checked by the caller on the host copy of the initial values).
bool lm_tirf_applies(const FitArgs &a, bool tirf_zero_held)
{
    return tirf_zero_held && a.model == IMFCS_MODEL_ACF_1D && a.npts <= kMaxPts && a.tol == 0.f && !a.cst &&
           (!a.linv || a.npts <= 96) && a.k == 3 && a.idx[0] == 0 && a.idx[1] == 1 && a.idx[2] == 4 &&
           a.np == IMFCS_NPARAM;
}

cudaError_t launch_lm_tirf(const FitArgs &a, int blocks, int threads, cudaStream_t s)
{
    const bool off = a.mc.rx != 0.f || a.mc.ry != 0.f;
    if (a.linv) {
        const size_t smem = (size_t)(threads / 32) * gls_warp_floats(a.npts) * sizeof(float);
        auto kern = off ? lm_tirf_kernel<true, true> : lm_tirf_kernel<false, true>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<blocks, threads, smem, s>>>(a);
    } else if (off) {
        lm_tirf_kernel<true, false><<<blocks, threads, 0, s>>>(a);
    } else {
        lm_tirf_kernel<false, false><<<blocks, threads, 0, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace imfcs
