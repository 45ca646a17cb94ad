// imfcs_fit.cu -- batched Levenberg-Marquardt fits, one warp per fit.
//
//   * FCS model (FCS_3p, java:13131-13408 / Gpufit ACF_1D, agpufitjni.cu:427-543)
//     weighted by 1/blocked variance over lags fitstart..fitend (standardFit,
//     java:10288-10471) or, for GLS, on the data and model transformed by
//     L^-1 of the regularised covariance (GLSFit, java:10622-10789).
//   * LINEAR_1D polynomial model (agpufitjni.cu:362-420).
//
// Lanes own fit points; J^T W J, J^T W r and chi^2 are warp reductions; the
// small K x K damped system is solved redundantly in every lane.  The grid is
// persistent: each warp strides over fits.  The solver stops on a small step
// (undamped Gauss-Newton step |h_i| <= 1e-7 |p_i| + 1e-5 sigma_i) once the
// residuals come from the FP64 model value, or when no step lowers chi^2 any
// more, or on the Gpufit criterion |dchi2| < tol max(1, chi2) when a
// tolerance is given through the reference fit API.
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
__device__ __forceinline__ double model_eval(const FitArgs &a, const ModelConst &mc, const ModelConstD &mcd,
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

    for (int fit = gw; fit < a.nfits; fit += nw) {
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
                // Newton steps on the FP64-residual gradient with the Hessian
                // of chi^2/2, H = -dg/dp, from forward differences (0.1 sigma)
                // of the FP32 gradient: converges in a few steps where
                // Gauss-Newton contracts only linearly on a non-zero residual.
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
                bool newton_done = false;
#pragma unroll 1
                for (int ni = 0; ni < 4; ni++) {
                    evaluate<KM>(a, mc, mcd, par, pard, yl, wl, xl, lane, sh_fj, sh_f64, sh_linv, s, c2, c3, true,
                                 yg, wg);
                    float hn[KM];
                    if (!isfinite(s.chi2) || !solve_scaled<KM>(H, s.g, a.k, 0.f, hn)) break;
                    bool conv = true;
#pragma unroll
                    for (int i = 0; i < KM; i++)
                        if (i < a.k) {
                            const float sig = rsqrtf(fmaxf(s.A[i * KM + i], 1e-30f));
                            conv = conv && (fabsf(hn[i]) <= 1e-7f * fabsf(par[a.idx[i]]) + 1e-5f * sig);
                            if (!(fabsf(hn[i]) <= 0.05f * sig)) ni = 4;   // not in the quadratic region
                        }
                    if (ni >= 4) break;
#pragma unroll
                    for (int i = 0; i < KM; i++)
                        if (i < a.k) {
                            pard[a.idx[i]] += (double)hn[i];
                            par[a.idx[i]] = (float)pard[a.idx[i]];
                        }
                    if (conv) { newton_done = true; break; }
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

template __global__ void lm_kernel<3, false>(FitArgs);
template __global__ void lm_kernel<5, false>(FitArgs);
template __global__ void lm_kernel<11, false>(FitArgs);
template __global__ void lm_kernel<3, true>(FitArgs);
template __global__ void lm_kernel<5, true>(FitArgs);
template __global__ void lm_kernel<11, true>(FitArgs);

size_t lm_smem_bytes(const FitArgs &a, int km, int warps)
{
    if (!a.linv) return 0;
    return (size_t)warps * ((size_t)a.npts * (a.npts + 1) / 2 + km * a.npts + 2 * a.npts + 2) * sizeof(float);
}

cudaError_t launch_lm(const FitArgs &a, int num_sms, cudaStream_t stream)
{
    if (a.nfits <= 0) return cudaSuccess;
    const bool big = a.npts > kMaxPts;
    if (big && a.linv) return cudaErrorInvalidValue;
    const int warps = 4;
    int km = a.k <= 3 ? 3 : (a.k <= 5 ? 5 : 11);
    size_t smem = lm_smem_bytes(a, km, warps);
    int blocks = (a.nfits + warps - 1) / warps;
    int cap = num_sms * 16;
    if (blocks > cap) blocks = cap;
    void (*kern)(FitArgs);
    if (km == 3) kern = big ? lm_kernel<3, true> : lm_kernel<3, false>;
    else if (km == 5) kern = big ? lm_kernel<5, true> : lm_kernel<5, false>;
    else kern = big ? lm_kernel<11, true> : lm_kernel<11, false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<blocks, warps * 32, smem, stream>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Pipeline glue: OLS data from the correlator outputs (double [pix][chanum])
// over lags fitstart..fitend, weights 1/var (java:10372).
// ---------------------------------------------------------------------------
__global__ void ols_prepare_kernel(int npix, int chanum, int fitstart, int npts, const double *acf,
                                   const double *var, float *y, float *w)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)npix * npts) return;
    size_t pix = i / npts;
    int p = (int)(i % npts);
    y[i] = (float)acf[pix * chanum + fitstart + p];
    w[i] = (float)(1.0 / var[pix * chanum + fitstart + p]);
}

// ---------------------------------------------------------------------------
// Fit epilogue (FP64, one thread per pixel): SI parameters, reduced chi^2 as
// the Java code reports it, the parameter covariance with commons-math's
// singularity threshold 1 (a singular covariance fails the fit exactly like
// the catch block of standardFit, java:10412, 10441), and the Bayes terms
// (java:10171-10207).
// ---------------------------------------------------------------------------


__device__ double det_lu(const double *ain, int n)
{
    // determinant by LU with partial pivoting (equal, up to rounding, to the
    // cofactor expansion of java:14752-14770)
    double a[IMFCS_NPARAM * IMFCS_NPARAM];
    for (int i = 0; i < n * n; i++) a[i] = ain[i];
    double det = 1.0;
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int r = c + 1; r < n; r++)
            if (fabs(a[r * n + c]) > fabs(a[p * n + c])) p = r;
        if (a[p * n + c] == 0.0) return 0.0;
        if (p != c) {
            for (int q = 0; q < n; q++) { double t = a[c * n + q]; a[c * n + q] = a[p * n + q]; a[p * n + q] = t; }
            det = -det;
        }
        det *= a[c * n + c];
        for (int r = c + 1; r < n; r++) {
            double f = a[r * n + c] / a[c * n + c];
            for (int q = c; q < n; q++) a[r * n + q] -= f * a[c * n + q];
        }
    }
    return det;
}

// Householder QR inverse with |R_ii| <= threshold -> singular.
__device__ bool qr_inverse_d(const double *ain, int k, double threshold, double *inv)
{
    double a[IMFCS_NPARAM * IMFCS_NPARAM], rdiag[IMFCS_NPARAM];
    for (int i = 0; i < k * k; i++) a[i] = ain[i];
    for (int minor = 0; minor < k; minor++) {
        double xn = 0.0;
        for (int r = minor; r < k; r++) xn += a[r * k + minor] * a[r * k + minor];
        double alpha = a[minor * k + minor] > 0 ? -sqrt(xn) : sqrt(xn);
        rdiag[minor] = alpha;
        if (alpha != 0.0) {
            a[minor * k + minor] -= alpha;
            for (int c = minor + 1; c < k; c++) {
                double ac = 0.0;
                for (int r = minor; r < k; r++) ac -= a[r * k + c] * a[r * k + minor];
                ac /= alpha * a[minor * k + minor];
                for (int r = minor; r < k; r++) a[r * k + c] -= ac * a[r * k + minor];
            }
        }
    }
    for (int i = 0; i < k; i++)
        if (!(fabs(rdiag[i]) > threshold)) return false;
    for (int col = 0; col < k; col++) {
        double y[IMFCS_NPARAM];
        for (int i = 0; i < k; i++) y[i] = (i == col) ? 1.0 : 0.0;
        for (int minor = 0; minor < k; minor++) {
            double dot = 0.0;
            for (int r = minor; r < k; r++) dot += y[r] * a[r * k + minor];
            dot /= rdiag[minor] * a[minor * k + minor];
            for (int r = minor; r < k; r++) y[r] += dot * a[r * k + minor];
        }
        for (int i = k - 1; i >= 0; i--) {
            y[i] /= rdiag[i];
            for (int r = 0; r < i; r++) y[r] -= y[i] * a[r * k + i];
        }
        for (int i = 0; i < k; i++) inv[i * k + col] = y[i];
    }
    return true;
}

__global__ void fit_epilogue_kernel(EpilogueArgs e)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= e.npix) return;
    const float *pi = e.par_int + (size_t)pix * IMFCS_NPARAM;
    int st = e.state[pix];
    bool ok = (st == IMFCS_STATE_CONVERGED) && (!e.pre_ok || e.pre_ok[pix]);
    double cov[IMFCS_NPARAM * IMFCS_NPARAM], jtj[IMFCS_NPARAM * IMFCS_NPARAM];
    const int k = e.k;
    for (int aa = 0; aa < k; aa++)
        for (int bb = 0; bb < k; bb++)
            jtj[aa * k + bb] = (double)e.hess[(size_t)pix * k * k + aa * k + bb] /
                               (param_unit(e.idx[aa]) * param_unit(e.idx[bb]));
    if (ok) ok = qr_inverse_d(jtj, k, 1.0, cov);
    for (int i = 0; i < k && ok; i++) ok = isfinite(cov[i * k + i]) && cov[i * k + i] > 0.0;
    float *fr = e.fitres + (size_t)pix * IMFCS_NPARAM;
    for (int i = 0; i < IMFCS_NPARAM; i++) {
        bool is_free = false;
        for (int q = 0; q < k; q++) is_free |= (e.idx[q] == i);
        fr[i] = (ok || !is_free) ? (float)((double)pi[i] * param_unit(i)) : nanf("");
    }
    if (e.chi2) e.chi2[pix] = ok ? (float)((double)e.chi2_raw[pix] / e.chi2_div) : nanf("");
    if (e.fitted) e.fitted[pix] = ok ? 1 : 0;
    if (e.logp) {
        // Bayes model-probability exponent (java:10171-10207):
        //   0.5 k ln(2 pi) + 0.5 ln det(cov) + logresid - ln(prod sigma * (2*200)^k)
        const double pi_j = 3.14159265359;
        double logresid, det, prodsig = 1.0;
        if (ok) {
            // unweighted residuals of the fitted lags (tres)
            double tres[kMaxChan];
            float par[IMFCS_NPARAM];
            for (int i = 0; i < IMFCS_NPARAM; i++) par[i] = pi[i];
            bool c2 = par[5] != 0.f, c3 = par[7] != 0.f;
            for (int i = 1; i < e.chanum; i++) {
                bool in = e.gls || (i >= e.fitstart && i <= e.fitend);
                double v = in ? (double)fcs_model_f(par, e.mc, e.lagtime[i], nullptr, c2, c3) : 0.0;
                tres[i - 1] = in ? e.acf[(size_t)pix * e.chanum + i] - v : 0.0;
            }
            if (!e.gls) {
                double rs = 0.0;
                for (int i = 1; i < e.chanum - 1; i++) rs += tres[i] * tres[i];   // from index 1 (java:10170)
                logresid = -0.5 * rs;
            } else {
                // tres^T covmats^-1 tres = |L^-1 tres|^2
                const int n = e.chanum - 1;
                const float *L = e.linv + (size_t)pix * n * (n + 1) / 2;
                double s = 0.0;
                for (int i = 0; i < n; i++) {
                    const float *row = L + (size_t)i * (i + 1) / 2;
                    double z = 0.0;
                    for (int c = 0; c <= i; c++) z += (double)row[c] * tres[c];
                    s += z * z;
                }
                logresid = -0.5 * s;
            }
            det = det_lu(cov, k);
            for (int i = 0; i < k; i++) prodsig *= sqrt(cov[i * k + i]);
        } else {
            // failed fit: ones (java:10441-10466) -> det of the all-ones matrix
            logresid = 0.0;
            for (int i = 1; i < e.chanum - 1; i++) logresid += 1.0;
            logresid *= -0.5;
            det = (k == 1) ? 1.0 : 0.0;
            prodsig = 1.0;
        }
        e.logp[pix] = 0.5 * k * log(2 * pi_j) + 0.5 * log(det) + logresid - log(prodsig * pow(400.0, k));
    }
}

__global__ void bayes_combine_kernel(int npix, const double *lp1, const double *lp2, float *prob)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    double m1 = exp(lp1[pix]), m2 = exp(lp2[pix]);
    double nrm = m1 + m2;
    prob[2 * pix] = (float)(m1 / nrm);
    prob[2 * pix + 1] = (float)(m2 / nrm);
}

cudaError_t launch_fit_epilogue(const EpilogueArgs &e, cudaStream_t stream)
{
    fit_epilogue_kernel<<<(e.npix + 127) / 128, 128, 0, stream>>>(e);
    return cudaGetLastError();
}
cudaError_t launch_ols_prepare(int npix, int chanum, int fitstart, int npts, const double *acf,
                               const double *var, float *y, float *w, cudaStream_t stream)
{
    size_t n = (size_t)npix * npts;
    ols_prepare_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(npix, chanum, fitstart, npts, acf, var, y, w);
    return cudaGetLastError();
}
cudaError_t launch_bayes_combine(int npix, const double *lp1, const double *lp2, float *prob,
                                 cudaStream_t stream)
{
    bayes_combine_kernel<<<(npix + 127) / 128, 128, 0, stream>>>(npix, lp1, lp2, prob);
    return cudaGetLastError();
}

}  // namespace imfcs
