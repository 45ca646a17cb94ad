// imfcs_lm_tirf.cu -- the LM fit of the plugin's default model, specialised:
// FCS_3p (java:13131-13408) with one component, no flow, no triplet, N, D and
// G free (the other parameters held at zero), OLS weights, up to kMaxPts
// points, step-mode stopping rule.  Same algorithm, stopping rules and FP32
// operation order as lm_kernel (imfcs_lm.cuh): phase 1 LM on FP32 model
// values, Newton finish with a forward-difference Hessian, FP32 then FP64
// residuals.  The model is evaluated from three scalars instead of the
// 11-parameter vector, so the parameters live in registers (no local-memory
// arrays indexed at run time) and the executed code is a few kilobytes --
// the generic kernel stalls on instruction fetch and local-memory loads.
#include "imfcs_lm.cuh"

namespace imfcs {

struct TirfC {
    float ax, ay, s2, inv_sz2, inv_norm;
    double axd, ayd, sd, szd, inv_normd;
    bool square;   // ax == ay: the two lateral factors coincide
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

// Model value and gradient (d/dN, d/dD; d/dG = 1) in FP32, internal units.
__device__ __noinline__ float tirf_f(float N, float D, float G, const TirfC &c, float tau, float &gN, float &gD)
{
    const float p0 = sqrtf(fmaf(4.f * D, tau, c.s2));
    const float inv_p0 = 1.f / p0;
    float Lx, dLx, Ly, dLy;
    tirf_lat(c.ax, p0, inv_p0, Lx, dLx);
    if (c.square) { Ly = Lx; dLy = dLx; }
    else tirf_lat(c.ay, p0, inv_p0, Ly, dLy);
    const float dp0 = 2.f * tau * inv_p0;
    const float lat = Lx * Ly * c.inv_norm;
    const float dlat = (dLx * Ly + Lx * dLy) * dp0 * c.inv_norm;
    const float psp = rsqrtf(fmaf(4.f * D * tau, c.inv_sz2, 1.f));
    const float dpsp = -2.f * tau * c.inv_sz2 * psp * psp * psp;
    const float a = lat * psp;
    const float da = dlat * psp + lat * dpsp;
    const float iN = 1.f / N;
    gN = -a * iN * iN;
    gD = iN * da;
    return __fmul_rn(a, iN) + G;
}

// FP64 model value (the precise residuals).
__device__ __noinline__ double tirf_d(double N, double D, double G, const TirfC &c, double tau)
{
    const double inv_sqrtpi = 0.56418958354775628695;
    const double p0 = sqrt(4.0 * D * tau + c.sd * c.sd);
    double u = c.axd / p0;
    const double lx = 2.0 * (p0 * inv_sqrtpi * expm1(-u * u) + c.axd * erf(u));
    double ly = lx;
    if (!c.square) {
        u = c.ayd / p0;
        ly = 2.0 * (p0 * inv_sqrtpi * expm1(-u * u) + c.ayd * erf(u));
    }
    const double lat = lx * ly * c.inv_normd;
    const double a1 = lat / sqrt(1.0 + 4.0 * D * tau / (c.szd * c.szd));
    return a1 / N + G;
}

struct Tirf3 {
    float A[9];
    float g[3];
    float chi2;      // FP32 phases
    double chi2d;    // FP64-residual evaluations
};

// One evaluation over the fit's points (warp): chi^2, J^T W J, J^T W r, with
// FP32 residuals, or (precise) residuals from the FP64 model value at the
// double parameters (Nd, Dd, Gd).  The FP32 phases use no FP64 operation:
// GB300 issues FP64 at 1/64 of the FP32 rate.
__device__ __noinline__ void tirf_eval(const TirfC &c, float N, float D, float G, double Nd, double Dd, double Gd,
                                       const float *yl, const float *wl, const float *xl, int n, int lane,
                                       bool precise, Tirf3 &s)
{
    float acc[9];
#pragma unroll
    for (int i = 0; i < 9; i++) acc[i] = 0.f;
    double c2acc = 0.0;
    float c2f = 0.f;
#pragma unroll
    for (int m = 0; m < kPtsPerLane; m++) {
        const int i = lane + 32 * m;
        if (i < n) {
            float gr[3];
            gr[2] = 1.f;
            const float f = tirf_f(N, D, G, c, xl[m], gr[0], gr[1]);
            const float w = wl[m];
            float r;
            if (precise) {
                const double rd = (double)yl[m] - tirf_d(Nd, Dd, Gd, c, (double)xl[m]);
                r = (float)rd;
                c2acc += (double)w * rd * rd;
            } else {
                r = yl[m] - f;
                c2f = fmaf(w * r, r, c2f);
            }
            int q = 0;
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int t = 0; t <= p; t++) acc[q++] += w * gr[p] * gr[t];
#pragma unroll
            for (int p = 0; p < 3; p++) acc[q++] += w * gr[p] * r;
        }
    }
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
    if (precise) {
        s.chi2d = warp_sum_d(c2acc);
        s.chi2 = (float)s.chi2d;
    } else {
        s.chi2 = warp_sum(c2f);
        s.chi2d = 0.0;
    }
}

__device__ __forceinline__ float tirf_sig(const Tirf3 &s, int i) { return rsqrtf(fmaxf(s.A[i * 3 + i], 1e-30f)); }

__global__ void __launch_bounds__(128) lm_tirf_kernel(FitArgs a)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int n = a.npts;
    const int gw = blockIdx.x * wpb + wib, nw = gridDim.x * wpb;
    TirfC c;
    c.ax = a.mc.ax; c.ay = a.mc.ay; c.s2 = a.mc.s * a.mc.s; c.inv_sz2 = 1.f / (a.mc.sz * a.mc.sz);
    c.inv_norm = a.mc.inv_norm;
    c.axd = a.mc.ax; c.ayd = a.mc.ay; c.sd = a.mc.s; c.szd = a.mc.sz; c.inv_normd = a.mc.inv_norm;
    c.square = a.mc.ay == a.mc.ax;
    float xl[kPtsPerLane];
#pragma unroll
    for (int m = 0; m < kPtsPerLane; m++) {
        const int i = lane + 32 * m;
        xl[m] = i < n ? __ldg(&a.x[i]) : 0.f;
    }
    for (int fit = a.counter ? lm_next_fit(a, 0, 0, lane) : gw; fit < a.nfits; fit = lm_next_fit(a, fit, nw, lane)) {
        if (a.todo && !__ldg(&a.todo[fit])) continue;
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
        Tirf3 s;
        tirf_eval(c, pf[0], pf[1], pf[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, s);
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
                        const float tol = precise ? 1e-7f * fabsf(pf[i]) + 1e-5f * sig : 1e-3f * sig;
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
                    tirf_eval(c, pnf[0], pnf[1], pnf[2], pnd[0], pnd[1], pnd[2], yl, wl, xl, n, lane, true, sn);
                    nprec++;
                    better = isfinite(sn.chi2d) && sn.chi2d < s.chi2d;
                } else {
#pragma unroll
                    for (int i = 0; i < 3; i++) pnf[i] = pf[i] + h[i];
                    tirf_eval(c, pnf[0], pnf[1], pnf[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, sn);
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
                    tirf_eval(c, pe[0], pe[1], pe[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, se);
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
                bool newton_done = false, left = false;
#pragma unroll 1
                for (int ni = 0; ni < 7 && !left; ni++) {
                    const bool fp64 = ni >= 3;
                    if (fp64) {
                        if (!precise) {
#pragma unroll
                            for (int i = 0; i < 3; i++) pd[i] = (double)pf[i];
                            precise = true;
                        }
                        tirf_eval(c, pf[0], pf[1], pf[2], pd[0], pd[1], pd[2], yl, wl, xl, n, lane, true, s);
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
                        if (small) ni = 2;
                        else tirf_eval(c, pf[0], pf[1], pf[2], 0.0, 0.0, 0.0, yl, wl, xl, n, lane, false, s);
                    }
                }
                if (newton_done) { state = IMFCS_STATE_CONVERGED; it++; break; }
                // otherwise LM on the FP64-residual model
                if (!precise) {
#pragma unroll
                    for (int i = 0; i < 3; i++) pd[i] = (double)pf[i];
                    precise = true;
                }
                tirf_eval(c, pf[0], pf[1], pf[2], pd[0], pd[1], pd[2], yl, wl, xl, n, lane, true, s);
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

// Whether a fit can take the specialised kernel: ACF model, OLS, step mode,
// shared constants without a window offset, N, D, G free in that order and
// every other parameter held at zero (tirf_zero_held: checked by the caller
// on the host copy of the initial values).
bool lm_tirf_applies(const FitArgs &a, bool tirf_zero_held)
{
    return tirf_zero_held && a.model == IMFCS_MODEL_ACF_1D && !a.linv && a.npts <= kMaxPts && a.tol == 0.f &&
           !a.cst && a.mc.rx == 0.f && a.mc.ry == 0.f && a.k == 3 && a.idx[0] == 0 && a.idx[1] == 1 &&
           a.idx[2] == 4 && a.np == IMFCS_NPARAM;
}

cudaError_t launch_lm_tirf(const FitArgs &a, int blocks, int threads, cudaStream_t s)
{
    lm_tirf_kernel<<<blocks, threads, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace imfcs
