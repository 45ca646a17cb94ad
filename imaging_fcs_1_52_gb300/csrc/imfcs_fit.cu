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

// lm_kernel (imfcs_lm.cuh): launchers in imfcs_lm{3,5,11}.cu
cudaError_t launch_lm_k3(const FitArgs &a, bool big, int blocks, int threads, size_t smem, cudaStream_t s);
cudaError_t launch_lm_k5(const FitArgs &a, bool big, int blocks, int threads, size_t smem, cudaStream_t s);
cudaError_t launch_lm_k11(const FitArgs &a, bool big, int blocks, int threads, size_t smem, cudaStream_t s);
// specialised kernel of the default fit (imfcs_lm_tirf.cu)
bool lm_tirf_applies(const FitArgs &a, bool tirf_zero_held);
cudaError_t launch_lm_tirf(const FitArgs &a, int blocks, int threads, cudaStream_t s);

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
    if (a.counter) {
        const cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(int), stream);
        if (e != cudaSuccess) return e;
    }
    if (lm_tirf_applies(a, a.tirf_zero_held != 0)) return launch_lm_tirf(a, blocks, warps * 32, stream);
    if (km == 3) return launch_lm_k3(a, big, blocks, warps * 32, smem, stream);
    if (km == 5) return launch_lm_k5(a, big, blocks, warps * 32, smem, stream);
    return launch_lm_k11(a, big, blocks, warps * 32, smem, stream);
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
