// imfcs_lm.cuh -- the batched Levenberg-Marquardt fit kernel (one warp per
// fit), instantiated per parameter-count bound KM in imfcs_lm3.cu,
// imfcs_lm5.cu and imfcs_lm11.cu (separate translation units so that the
// heavily unrolled variants compile in parallel); launched through their
// launchers by imfcs_fit.cu, which describes the algorithm.
#pragma once

#include <math.h>

#include "imfcs_internal.cuh"
#include "imfcs_args.h"

namespace imfcs {

constexpr int kMaxPts = 160;
constexpr int kPtsPerLane = kMaxPts / 32;



template <int KM>
struct LMState {
    float A[KM * KM];
    float g[KM];
    double chi2;
};

__device__ __forceinline__ ModelConst load_consts(const float *c)
{
    // SI -> internal (um)
    ModelConst m;
    m.ax = c[0] * 1e6f; m.ay = c[1] * 1e6f; m.s = c[2] * 1e6f; m.sz = c[3] * 1e6f;
    m.rx = c[4] * 1e6f; m.ry = c[5] * 1e6f;
    float fo = c[6] * 1e12f;
    m.inv_norm = fo / (4.f * m.ax * m.ay * m.ax * m.ay);
    m.q2 = c[7]; m.q3 = c[8];
    return m;
}

__device__ __forceinline__ ModelConstD to_double(const ModelConst &m)
{
    ModelConstD d;
    d.ax = m.ax; d.ay = m.ay; d.s = m.s; d.sz = m.sz; d.rx = m.rx; d.ry = m.ry;
    d.inv_norm = m.inv_norm; d.q2 = m.q2; d.q3 = m.q3;
    return d;
}

// Model value and gradient w.r.t. the free parameters at x.  precise: the
// value comes from the FP64 model (ACF model); the gradient is always FP32.
template <int KM>
__device__ __noinline__ double model_eval(const FitArgs &a, const ModelConst &mc, const ModelConstD &mcd,
                                             const float *par, const double *pard, float x, float *gfree,
                                             bool c2, bool c3, bool precise)
{
    if (a.model == IMFCS_MODEL_ACF_1D) {
        float g[IMFCS_NPARAM];
        float v = fcs_model_f(par, mc, x, g, c2, c3);
#pragma unroll
        for (int i = 0; i < KM; i++)
            if (i < a.k) gfree[i] = g[a.idx[i]];
        return precise ? fcs_model_value_d(pard, mcd, (double)x, c2, c3) : (double)v;
    } else {
        float g[IMFCS_NPARAM];
        double v = 0.0, pw = 1.0;
        for (int i = 0; i < a.np; i++) { g[i] = (float)pw; v = fma(pard[i], pw, v); pw *= (double)x; }
#pragma unroll
        for (int i = 0; i < KM; i++)
            if (i < a.k) gfree[i] = g[a.idx[i]];
        return v;
    }
}

// One evaluation: chi^2, A = J^T W J, g = J^T W r over all points (warp).
// Per-lane partial sums in FP32 (a handful of points each), warp reduction in
// FP64; chi^2 and the residuals in FP64.  For GLS the model vector and the
// Jacobian are first transformed by L^-1 held in shared memory (packed lower
// triangle); y then holds the transformed data.
template <int KM>
__device__ __forceinline__ void accumulate_point(float *acc, double &c2acc, float &c2f, const float *gr, double rd,
                                                 float w, bool precise)
{
    float r = (float)rd;
    int q = 0;
#pragma unroll
    for (int p = 0; p < KM; p++)
#pragma unroll
        for (int t = 0; t <= p; t++) acc[q++] += w * gr[p] * gr[t];
#pragma unroll
    for (int p = 0; p < KM; p++) acc[q++] += w * gr[p] * r;
    if (precise) c2acc += (double)w * rd * rd;
    else c2f = fmaf(w * r, r, c2f);       // FP32 phase: a few points per lane
}

// yg/wg (non-null): the fit's data are read from global memory point by point
// (fits with more than kMaxPts points, no GLS transform).
template <int KM>
__device__ __noinline__ void evaluate(const FitArgs &a, const ModelConst &mc, const ModelConstD &mcd, const float *par,
                         const double *pard, const float *yl, const float *wl, const float *xl, int lane,
                         float *sh_fj, double *sh_f64, const float *sh_linv, LMState<KM> &s, bool c2,
                         bool c3, bool precise, const float *yg = nullptr, const float *wg = nullptr)
{
    constexpr int NACC = KM * (KM + 1) / 2 + KM;
    float acc[NACC];
    double c2acc = 0.0;
    float c2f = 0.f;
#pragma unroll
    for (int i = 0; i < NACC; i++) acc[i] = 0.f;
    const int n = a.npts;
    if (yg) {
        for (int i = lane; i < n; i += 32) {
            float gr[KM];
            double f = model_eval<KM>(a, mc, mcd, par, pard, __ldg(&a.x[i]), gr, c2, c3, precise);
            accumulate_point<KM>(acc, c2acc, c2f, gr, (double)__ldg(&yg[i]) - f, wg ? __ldg(&wg[i]) : 1.f, precise);
        }
    } else if (!sh_linv) {
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            int i = lane + 32 * m;
            if (i < n) {
                float gr[KM];
                double f = model_eval<KM>(a, mc, mcd, par, pard, xl[m], gr, c2, c3, precise);
                if (precise) {
                    accumulate_point<KM>(acc, c2acc, c2f, gr, (double)yl[m] - f, wl[m], true);
                } else {
                    // FP32 phase: FP32 residual, no FP64 operation per point
                    accumulate_point<KM>(acc, c2acc, c2f, gr, (double)(yl[m] - (float)f), wl[m], false);
                }
            }
        }
    } else {
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            int i = lane + 32 * m;
            if (i < n) {
                float gr[KM];
                double f = model_eval<KM>(a, mc, mcd, par, pard, xl[m], gr, c2, c3, precise);
                sh_f64[i] = f;
#pragma unroll
                for (int p = 0; p < KM; p++) sh_fj[p * n + i] = (p < a.k) ? gr[p] : 0.f;
            }
        }
        __syncwarp();
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            int i = lane + 32 * m;
            if (i < n) {
                const float *row = sh_linv + (size_t)i * (i + 1) / 2;
                double f = 0.0;
                float gr[KM];
#pragma unroll
                for (int p = 0; p < KM; p++) gr[p] = 0.f;
                for (int c = 0; c <= i; c++) {
                    float l = row[c];
                    f = fma((double)l, sh_f64[c], f);
#pragma unroll
                    for (int p = 0; p < KM; p++) gr[p] = fmaf(l, sh_fj[p * n + c], gr[p]);
                }
                double rd = (double)yl[m] - f;
                float r = (float)rd;
                int q = 0;
#pragma unroll
                for (int p = 0; p < KM; p++)
#pragma unroll
                    for (int t = 0; t <= p; t++) acc[q++] += gr[p] * gr[t];
#pragma unroll
                for (int p = 0; p < KM; p++) acc[q++] += gr[p] * r;
                c2acc += rd * rd;
            }
        }
        __syncwarp();
    }
    int q = 0;
#pragma unroll
    for (int p = 0; p < KM; p++)
#pragma unroll
        for (int t = 0; t <= p; t++) {
            float v = warp_sum(acc[q++]);
            s.A[p * KM + t] = v;
            s.A[t * KM + p] = v;
        }
#pragma unroll
    for (int p = 0; p < KM; p++) s.g[p] = warp_sum(acc[q++]);
    s.chi2 = precise ? warp_sum_d(c2acc + (double)c2f) : (double)warp_sum(c2f + (float)c2acc);
}

// (A + lambda diag(A)) h = g, solved in FP32 on the Jacobi-scaled system
// (unit diagonal), which keeps the Cholesky stable for strongly correlated
// parameters.  Accuracy of the fixed point is set by g, not by this solve.
template <int KM>
__device__ __forceinline__ bool solve_scaled(const float *A, const float *g, int k, float lambda, float *h)
{
    float sc[KM], L[KM * KM];
#pragma unroll
    for (int i = 0; i < KM; i++) sc[i] = (i < k) ? rsqrtf(fmaxf(A[i * KM + i], 1e-30f)) : 0.f;
#pragma unroll
    for (int r = 0; r < KM; r++)
#pragma unroll
        for (int c = 0; c < KM; c++) L[r * KM + c] = A[r * KM + c] * sc[r] * sc[c];
#pragma unroll
    for (int i = 0; i < KM; i++)
        if (i < k) L[i * KM + i] = 1.f + lambda;
#pragma unroll
    for (int c = 0; c < KM; c++) {
        if (c >= k) break;
        float d = L[c * KM + c];
#pragma unroll
        for (int m = 0; m < KM; m++)
            if (m < c) d -= L[c * KM + m] * L[c * KM + m];
        if (!(d > 0.f) || !isfinite(d)) return false;
        d = sqrtf(d);
        L[c * KM + c] = d;
        float id = 1.f / d;
#pragma unroll
        for (int r = 0; r < KM; r++) {
            if (r <= c || r >= k) continue;
            float sum = L[r * KM + c];
#pragma unroll
            for (int m = 0; m < KM; m++)
                if (m < c) sum -= L[r * KM + m] * L[c * KM + m];
            L[r * KM + c] = sum * id;
        }
    }
    float yv[KM], z[KM];
#pragma unroll
    for (int r = 0; r < KM; r++) {
        if (r >= k) { yv[r] = 0.f; continue; }
        float sum = g[r] * sc[r];
#pragma unroll
        for (int m = 0; m < KM; m++)
            if (m < r) sum -= L[r * KM + m] * yv[m];
        yv[r] = sum / L[r * KM + r];
    }
#pragma unroll
    for (int r = KM - 1; r >= 0; r--) {
        if (r >= k) { z[r] = 0.f; continue; }
        float sum = yv[r];
#pragma unroll
        for (int m = 0; m < KM; m++)
            if (m > r && m < k) sum -= L[m * KM + r] * z[m];
        z[r] = sum / L[r * KM + r];
    }
#pragma unroll
    for (int r = 0; r < KM; r++) h[r] = z[r] * sc[r];
    return true;
}

// Next fit of a warp: a static stride over the fits, or, with a work counter,
// the next unclaimed fit (so that warps whose fits converge early take more).
__device__ __forceinline__ int lm_next_fit(const FitArgs &a, int fit, int nw, int lane)
{
    if (!a.counter) return fit + nw;
    int f = 0;
    if (lane == 0) f = atomicAdd(a.counter, 1);
    return __shfl_sync(0xffffffffu, f, 0);
}

template <int KM, bool BIG>
__global__ void __launch_bounds__(128) lm_kernel(FitArgs a)
{
    extern __shared__ float fsh[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int n = a.npts;
    const int linv_len = n * (n + 1) / 2;
    // per warp (GLS only): L^-1 (float), Jacobian (float), model values (double)
    const size_t per_warp = (size_t)linv_len + KM * n + 2 * n + 2;
    float *sh_linv = a.linv ? fsh + (size_t)wib * per_warp : nullptr;
    float *sh_fj = a.linv ? sh_linv + linv_len : nullptr;
    double *sh_f64 = nullptr;
    if (a.linv) {
        size_t off = ((size_t)(sh_fj + KM * n - fsh) + 1) & ~(size_t)1;   // 8-byte aligned
        sh_f64 = (double *)(fsh + off);
    }
    const int gw = blockIdx.x * wpb + wib, nw = gridDim.x * wpb;

    float xl[kPtsPerLane];
#pragma unroll
    for (int m = 0; m < kPtsPerLane; m++) {
        int i = lane + 32 * m;
        xl[m] = (!BIG && i < n) ? __ldg(&a.x[i]) : 0.f;
    }

    for (int fit = a.counter ? lm_next_fit(a, 0, 0, lane) : gw; fit < a.nfits; fit = lm_next_fit(a, fit, nw, lane)) {
        if (a.todo && !__ldg(&a.todo[fit])) continue;
        float yl[kPtsPerLane], wl[kPtsPerLane];
#pragma unroll
        for (int m = 0; m < kPtsPerLane; m++) {
            int i = lane + 32 * m;
            bool in = !BIG && i < n;
            yl[m] = in ? __ldg(&a.y[(size_t)fit * n + i]) : 0.f;
            wl[m] = in ? (a.w ? __ldg(&a.w[(size_t)fit * n + i]) : 1.f) : 0.f;
        }
        const float *yg = BIG ? a.y + (size_t)fit * n : nullptr;
        const float *wg = (BIG && a.w) ? a.w + (size_t)fit * n : nullptr;
        if (sh_linv) {
            const float *src = a.linv + (size_t)fit * linv_len;
            for (int i = lane; i < linv_len; i += 32) sh_linv[i] = __ldg(&src[i]);
            __syncwarp();
        }
        const ModelConst mc = a.cst ? load_consts(a.cst + (size_t)fit * IMFCS_NCONST) : a.mc;
        const ModelConstD mcd = to_double(mc);
        float par[IMFCS_NPARAM];
        double pard[IMFCS_NPARAM];
        const float *ip = a.init + (size_t)fit * a.init_stride;
        for (int i = 0; i < a.np; i++) { par[i] = __ldg(&ip[i]); pard[i] = par[i]; }
        bool c2 = false, c3 = false;
        if (a.model == IMFCS_MODEL_ACF_1D) {
            bool f2free = false, f3free = false;
            for (int i = 0; i < a.k; i++) {
                f2free |= (a.idx[i] == 5 || a.idx[i] == 6);
                f3free |= (a.idx[i] == 7 || a.idx[i] == 8);
            }
            c2 = par[5] != 0.f || f2free;
            c3 = par[7] != 0.f || f3free;
        }
        // Gpufit mode (tol > 0): FP32 model values throughout, Gpufit's stop
        // rule.  Step mode, ACF model: phase 1 with FP32 model values until
        // the Gauss-Newton step is below 1e-3 sigma (or no step lowers chi^2
        // up to lambda 1e6); phase 2 with residuals from the FP64 model value
        // until the step is below 1e-5 sigma + 1e-7 |p| (or no step lowers
        // chi^2 up to lambda 1e10).  The linear model is FP64 throughout.
        const bool gpufit = a.tol > 0.f;
        bool precise = a.model != IMFCS_MODEL_ACF_1D;
        LMState<KM> s;
        evaluate<KM>(a, mc, mcd, par, pard, yl, wl, xl, lane, sh_fj, sh_f64, sh_linv, s, c2, c3, precise, yg, wg);
        int state = IMFCS_STATE_MAX_ITERATIONS, it = 0, nprec = 0;
        float lambda = 1e-3f;
        if (!isfinite(s.chi2)) state = IMFCS_STATE_SINGULAR_HESSIAN;
        else if (a.k == 0) state = IMFCS_STATE_CONVERGED;
        for (it = 0; state == IMFCS_STATE_MAX_ITERATIONS && it < a.max_iter; it++) {
            float h[KM];
            bool to_precise = false;
            if (!gpufit) {
                float hg[KM];
                if (solve_scaled<KM>(s.A, s.g, a.k, 0.f, hg)) {
                    bool conv = true;
#pragma unroll
                    for (int i = 0; i < KM; i++)
                        if (i < a.k) {
                            float sig = rsqrtf(fmaxf(s.A[i * KM + i], 1e-30f));
                            float tol = precise ? 1e-7f * fabsf(par[a.idx[i]]) + 1e-5f * sig : 1e-3f * sig;
                            conv = conv && (fabsf(hg[i]) <= tol);
                        }
                    if (conv) {
                        if (precise) { state = IMFCS_STATE_CONVERGED; break; }
                        to_precise = true;
                    }
                }
            }
            if (!to_precise) {
                if (!solve_scaled<KM>(s.A, s.g, a.k, lambda, h)) {
                    lambda *= 10.f;
                    if (lambda > 1e15f) { state = IMFCS_STATE_SINGULAR_HESSIAN; break; }
                    continue;
                }
                double pnd[IMFCS_NPARAM];
                float pnf[IMFCS_NPARAM];
                for (int i = 0; i < a.np; i++) pnd[i] = pard[i];
#pragma unroll
                for (int i = 0; i < KM; i++)
                    if (i < a.k) pnd[a.idx[i]] = pard[a.idx[i]] + (double)h[i];
                for (int i = 0; i < a.np; i++) pnf[i] = (float)pnd[i];
                LMState<KM> sn;
                evaluate<KM>(a, mc, mcd, pnf, pnd, yl, wl, xl, lane, sh_fj, sh_f64, sh_linv, sn, c2, c3, precise,
                             yg, wg);
                if (precise && a.model == IMFCS_MODEL_ACF_1D) nprec++;
                const bool finite = isfinite(sn.chi2);
                const bool better = finite && sn.chi2 < s.chi2;
                if (gpufit) {
                    // Gpufit semantics (agpufitjni.cu:2289-2320, 2458-2487);
                    // the ACF model then gets the FP64-residual finish below
                    bool found = finite && fabs(sn.chi2 - s.chi2) < (double)a.tol * fmax(1.0, sn.chi2);
                    if (better) {
                        for (int i = 0; i < a.np; i++) { pard[i] = pnd[i]; par[i] = pnf[i]; }
                        s = sn;
                        lambda *= 0.1f;
                    } else {
                        lambda *= 10.f;
                    }
                    if (found || lambda > 1e30f) {
                        if (a.model == IMFCS_MODEL_ACF_1D && !precise) {
                            to_precise = true;
                        } else {
                            state = IMFCS_STATE_CONVERGED;
                            it++;
                            break;
                        }
                    }
                    if (!to_precise) continue;
                }
                if (gpufit) {
                    // handled above
                } else if (better) {
                    for (int i = 0; i < a.np; i++) { pard[i] = pnd[i]; par[i] = pnf[i]; }
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
                // Newton finish with the Hessian of chi^2/2, H = -dg/dp, from
                // forward differences (0.1 sigma) of the FP32 gradient:
                // Gauss-Newton contracts only linearly on a non-zero residual.
                // (a) steps on the FP32-residual gradient to its stationary
                //     point (cheap); (b) steps on the gradient of residuals
                //     from the FP64 model value until the step is below
                //     1e-4 sigma + 1e-7 |p| -- usually the first one, so one
                //     FP64 evaluation per fit; the remaining error is about
                //     the Hessian's relative error times that step.
                float H[KM * KM];
#pragma unroll
                for (int i = 0; i < KM * KM; i++) H[i] = 0.f;
                for (int i = 0; i < a.k; i++) {
                    float sgi = 0.f;
#pragma unroll
                    for (int q = 0; q < KM; q++)
                        if (q == i) sgi = rsqrtf(fmaxf(s.A[q * KM + q], 1e-30f));
                    const float eps = 0.1f * sgi;
                    float pe[IMFCS_NPARAM];
                    double pde[IMFCS_NPARAM];
                    for (int q = 0; q < a.np; q++) { pe[q] = par[q]; pde[q] = pard[q]; }
                    pde[a.idx[i]] += (double)eps;
                    pe[a.idx[i]] = (float)pde[a.idx[i]];
                    const float de = (float)(pde[a.idx[i]] - pard[a.idx[i]]);
                    LMState<KM> se;
                    evaluate<KM>(a, mc, mcd, pe, pde, yl, wl, xl, lane, sh_fj, sh_f64, sh_linv, se, c2, c3, false,
                                 yg, wg);
#pragma unroll
                    for (int r = 0; r < KM; r++)
#pragma unroll
                        for (int q = 0; q < KM; q++)
                            if (q == i) H[r * KM + q] = (s.g[r] - se.g[r]) / de;
                }
#pragma unroll
                for (int r = 0; r < KM; r++)
#pragma unroll
                    for (int q = 0; q < r; q++) {
                        const float v = 0.5f * (H[r * KM + q] + H[q * KM + r]);
                        H[r * KM + q] = v;
                        H[q * KM + r] = v;
                    }
                bool newton_done = false, left = false;
#pragma unroll 1
                for (int ni = 0; ni < 7 && !left; ni++) {
                    const bool fp64 = ni >= 3;   // (a) 3 FP32 steps at most, then (b)
                    if (fp64) {
                        evaluate<KM>(a, mc, mcd, par, pard, yl, wl, xl, lane, sh_fj, sh_f64, sh_linv, s, c2, c3, true,
                                     yg, wg);
                        if (!isfinite(s.chi2)) { left = true; break; }
                    }
                    float hn[KM];
                    if (!solve_scaled<KM>(H, s.g, a.k, 0.f, hn)) { left = true; break; }
                    bool small = true;
#pragma unroll
                    for (int i = 0; i < KM; i++)
                        if (i < a.k) {
                            const float sig = rsqrtf(fmaxf(s.A[i * KM + i], 1e-30f));
                            if (!(fabsf(hn[i]) <= 0.05f * sig)) left = true;   // not in the quadratic region
                            small = small && (fabsf(hn[i]) <= 1e-4f * sig + (fp64 ? 1e-7f * fabsf(par[a.idx[i]]) : 0.f));
                        }
                    if (left) break;
#pragma unroll
                    for (int i = 0; i < KM; i++)
                        if (i < a.k) {
                            pard[a.idx[i]] += (double)hn[i];
                            par[a.idx[i]] = (float)pard[a.idx[i]];
                        }
                    if (fp64 && small) { newton_done = true; break; }
                    if (!fp64) {
                        if (small) ni = 2;       // at the FP32 stationary point: go to (b)
                        else
                            evaluate<KM>(a, mc, mcd, par, pard, yl, wl, xl, lane, sh_fj, sh_f64, sh_linv, s, c2, c3,
                                         false, yg, wg);
                    }
                }
                if (newton_done) { state = IMFCS_STATE_CONVERGED; it++; break; }
                // otherwise: Levenberg-Marquardt on the FP64-residual model
                precise = true;
                evaluate<KM>(a, mc, mcd, par, pard, yl, wl, xl, lane, sh_fj, sh_f64, sh_linv, s, c2, c3, true,
                             yg, wg);
                lambda = 1e-3f;
            }
        }
        if (lane == 0) {
            for (int i = 0; i < a.np; i++) a.out_par[(size_t)fit * a.out_stride + i] = (float)pard[i];
            if (a.out_chi2) a.out_chi2[fit] = (float)s.chi2;
            if (a.out_state) a.out_state[fit] = state;
            if (a.out_iter) a.out_iter[fit] = it;
            if (a.out_hess)
                for (int i = 0; i < a.k * a.k; i++)
                    a.out_hess[(size_t)fit * a.k * a.k + i] = s.A[(i / a.k) * KM + (i % a.k)];
        }
        __syncwarp();
    }
}

}  // namespace imfcs
