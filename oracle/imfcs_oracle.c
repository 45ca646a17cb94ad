/*
 * imfcs_oracle.c -- FP64 CPU restatement of the Imaging_FCS 1.52 Java CPU
 * correlation-and-fit path.  TEST INFRASTRUCTURE ONLY (see imfcs_oracle.h).
 *
 * Compile with -ffp-contract=off so that x86-64 and aarch64 hosts give the
 * same rounding as the Java code (no fused multiply-add contraction).
 *
 * The Levenberg-Marquardt solver below stands in for commons-math3 3.6.1's
 * LevenbergMarquardtOptimizer (not vendored in the reference; the plugin
 * reaches it through AbstractCurveFitter.getOptimizer(), e.g. java:10343).
 * It restates the published Levenberg-Marquardt method with Marquardt/More
 * diagonal scaling and Nielsen's damping update; parity is on the converged
 * minimum, not on the iteration path.
 */
#include "imfcs_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQR(x) ((x) * (x))

/* ------------------------------------------------------------------------ */
/* Lag tables: java:7340-7346 (chanum), java:7391-7424 (lag, samp, mtab).    */
/* ------------------------------------------------------------------------ */
int imfcs_o_chanum(int p, int q) { return (int)(p + (q - 1) * (double)p / 2 + 1); }

void imfcs_o_lag_tables(int p, int q, int num, int *lag, double *samp, double *mtab)
{
    int base = p, hbase = p / 2, lagnum = q;
    int chanum = imfcs_o_chanum(p, q);
    for (int x = 0; x <= hbase; x++) lag[x] = x;
    for (int x = 1; x <= lagnum; x++)
        for (int y = 1; y <= hbase; y++)
            lag[x * hbase + y] = (int)(pow(2, x - 1) * y + (base / 4) * pow(2, x));
    for (int x = 0; x <= base; x++) samp[x] = 1;
    for (int x = 2; x <= lagnum; x++)
        for (int y = 1; y <= hbase; y++) samp[x * hbase + y] = pow(2, x - 1);
    for (int x = 0; x < chanum; x++) mtab[x] = (int)floor((num - lag[x]) / samp[x]);
}

/* ------------------------------------------------------------------------ */
/* Intensity: getIntensity java:9651-9678, calcIntensityTrace 9822-9855.    */
/* ------------------------------------------------------------------------ */
static inline int bg_at(const int *bgr, int width, int x, int y, int bckg)
{
    return bgr ? bgr[(size_t)y * width + x] : bckg;
}

void imfcs_o_get_intensity(const uint16_t *stack, int width, int height, int first, int num,
                           int px, int py, int binx, int biny, int bckg, const int *bgr,
                           double *out)
{
    size_t fsz = (size_t)width * height;
    out[0] = 0.0;
    for (int x = 1; x <= num; x++) {
        const uint16_t *fr = stack + (size_t)(first + x - 1) * fsz;
        double acc = 0.0;
        for (int i = 0; i < binx; i++)
            for (int k = 0; k < biny; k++)
                acc += (double)((int)fr[(size_t)(py + k) * width + px + i] -
                                bg_at(bgr, width, px + i, py + k, bckg));
        out[x] = acc;
    }
}

/* bgx, bgy: the window whose background-image pixels are subtracted.  The
 * reference subtracts the first (direct) window's values from both traces of
 * a cross-correlation (bckg1 and bckg2 both read bgrmean[ipx1 + i][ipy1 + k],
 * java:9842-9845); with a scalar background the two coincide. */
void imfcs_o_intensity_trace(const uint16_t *stack, int width, int height, int first, int num,
                             int px, int py, int bgx, int bgy, int binx, int biny, int bckg,
                             const int *bgr, int nopit, double frametime, double *trace,
                             double *trace_time)
{
    size_t fsz = (size_t)width * height;
    int ave = (int)floor((double)num / nopit);
    (void)height;
    for (int x = 0; x < nopit; x++) {
        int sum = 0; /* Java int accumulator and int division (java:9852) */
        for (int i = 0; i < binx; i++)
            for (int k = 0; k < biny; k++)
                for (int y = first + x * ave; y <= first + (x + 1) * ave - 1; y++)
                    sum += (int)stack[(size_t)y * fsz + (size_t)(py + k) * width + px + i] -
                           bg_at(bgr, width, bgx + i, bgy + k, bckg);
        trace_time[x] = frametime * (x + 0.5) * ave;
        trace[x] = (double)(sum / ave);
    }
}

/* ------------------------------------------------------------------------ */
/* Small dense linear algebra (FP64).                                        */
/* ------------------------------------------------------------------------ */
/* Cholesky of SPD a (k x k, row-major, overwritten by L). 0 on success. */
static int chol_inplace(double *a, int k)
{
    for (int j = 0; j < k; j++) {
        double d = a[j * k + j];
        for (int m = 0; m < j; m++) d -= a[j * k + m] * a[j * k + m];
        if (!(d > 0.0) || !isfinite(d)) return 1;
        d = sqrt(d);
        a[j * k + j] = d;
        for (int i = j + 1; i < k; i++) {
            double s = a[i * k + j];
            for (int m = 0; m < j; m++) s -= a[i * k + m] * a[j * k + m];
            a[i * k + j] = s / d;
        }
        for (int i = 0; i < j; i++) a[i * k + j] = 0.0;
    }
    return 0;
}

static void chol_solve(const double *l, int k, const double *b, double *x)
{
    double y[64];
    for (int i = 0; i < k; i++) {
        double s = b[i];
        for (int m = 0; m < i; m++) s -= l[i * k + m] * y[m];
        y[i] = s / l[i * k + i];
    }
    for (int i = k - 1; i >= 0; i--) {
        double s = y[i];
        for (int m = i + 1; m < k; m++) s -= l[m * k + i] * x[m];
        x[i] = s / l[i * k + i];
    }
}

/* Householder QR inverse of a square matrix with a singularity threshold on
 * |R_ii|, as used for the parameter covariance (commons-math
 * getCovariances(1), java:10412, 10727).  Returns 0 on success. */
static int qr_inverse(const double *a_in, int k, double threshold, double *inv)
{
    double a[64 * 64], rdiag[64];
    memcpy(a, a_in, sizeof(double) * k * k);
    /* column-wise Householder on a (k x k) */
    for (int minor = 0; minor < k; minor++) {
        double xnorm = 0.0;
        for (int r = minor; r < k; r++) xnorm += a[r * k + minor] * a[r * k + minor];
        double alpha = a[minor * k + minor] > 0 ? -sqrt(xnorm) : sqrt(xnorm);
        rdiag[minor] = alpha;
        if (alpha != 0.0) {
            a[minor * k + minor] -= alpha;
            for (int c = minor + 1; c < k; c++) {
                double alphac = 0.0;
                for (int r = minor; r < k; r++) alphac -= a[r * k + c] * a[r * k + minor];
                alphac /= alpha * a[minor * k + minor];
                for (int r = minor; r < k; r++) a[r * k + c] -= alphac * a[r * k + minor];
            }
        }
    }
    for (int i = 0; i < k; i++)
        if (fabs(rdiag[i]) <= threshold) return 1;
    /* solve A X = I column by column: apply Q^T then back substitute */
    for (int col = 0; col < k; col++) {
        double y[64];
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
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Levenberg-Marquardt (FP64).  Minimises sum_i w_i (y_i - f_i(p))^2.        */
/* ------------------------------------------------------------------------ */
typedef void (*lm_model_fn)(const double *p, double *f, double *jac, void *ctx);

typedef struct {
    double chi2;
    int iters;
    int evals;
} lm_info;

/* jw (optional, n x k) receives the weighted Jacobian sqrt(w)*df/dp at the
 * optimum.  Returns 0 on convergence, 1 on max iterations, 2 on failure. */
static int lm_solve(lm_model_fn fn, void *ctx, int n, int k, const double *y,
                    const double *w, double *p, int max_iter, lm_info *info, double *jw)
{
    const double ftol = 1e-10, xtol = 1e-10, gtol = 1e-10;
    double *f = (double *)malloc(sizeof(double) * n * (2 + 2 * k));
    double *jac = f + n, *fn_new = jac + (size_t)n * k, *jac_new = fn_new + n;
    double a[64 * 64], l[64 * 64], g[64], h[64], pn[64], dg[64];
    double mu = 0.0, nu = 2.0, chi2 = 0.0;
    int status = 1, it = 0, evals = 0;

    fn(p, f, jac, ctx);
    evals++;
    for (int j = 0; j < k; j++) dg[j] = 0.0;

    for (it = 0; it < max_iter; it++) {
        /* residuals, A = J^T W J, g = J^T W r (r = y - f, J = df/dp) */
        chi2 = 0.0;
        for (int j = 0; j < k; j++) { g[j] = 0.0; for (int m = 0; m < k; m++) a[j * k + m] = 0.0; }
        for (int i = 0; i < n; i++) {
            double wi = w ? w[i] : 1.0, r = y[i] - f[i];
            if (!isfinite(r) || !isfinite(wi)) { status = 2; goto done; }
            chi2 += wi * r * r;
            for (int j = 0; j < k; j++) {
                double jj = jac[(size_t)i * k + j];
                g[j] += wi * jj * r;
                for (int m = 0; m <= j; m++) a[j * k + m] += wi * jj * jac[(size_t)i * k + m];
            }
        }
        for (int j = 0; j < k; j++)
            for (int m = j + 1; m < k; m++) a[j * k + m] = a[m * k + j];
        for (int j = 0; j < k; j++) {
            double cn = sqrt(a[j * k + j]);
            if (cn > dg[j]) dg[j] = cn;
            if (dg[j] == 0.0) dg[j] = 1.0;
        }
        if (it == 0) {
            double mx = 0.0;
            for (int j = 0; j < k; j++) mx = fmax(mx, a[j * k + j] / (dg[j] * dg[j]));
            mu = 1e-3 * mx;
            if (!(mu > 0)) mu = 1e-3;
        }
        /* gradient test (cosine of residual and Jacobian columns) */
        {
            double gmax = 0.0, rn = sqrt(chi2);
            for (int j = 0; j < k; j++) {
                double cn = sqrt(a[j * k + j]);
                if (cn > 0 && rn > 0) gmax = fmax(gmax, fabs(g[j]) / (cn * rn));
            }
            if (gmax <= gtol) { status = 0; goto done; }
        }
        /* inner loop: find an acceptable step */
        for (;;) {
            for (int j = 0; j < k * k; j++) l[j] = a[j];
            for (int j = 0; j < k; j++) l[j * k + j] += mu * dg[j] * dg[j];
            if (chol_inplace(l, k)) {
                mu *= nu; nu *= 2.0;
                if (mu > 1e300) { status = 2; goto done; }
                continue;
            }
            chol_solve(l, k, g, h);
            double pnorm = 0.0, hnorm = 0.0;
            for (int j = 0; j < k; j++) {
                pn[j] = p[j] + h[j];
                pnorm += SQR(dg[j] * p[j]);
                hnorm += SQR(dg[j] * h[j]);
            }
            pnorm = sqrt(pnorm); hnorm = sqrt(hnorm);
            fn(pn, fn_new, jac_new, ctx);
            evals++;
            double chi2n = 0.0;
            int finite = 1;
            for (int i = 0; i < n; i++) {
                double wi = w ? w[i] : 1.0, r = y[i] - fn_new[i];
                if (!isfinite(r)) { finite = 0; break; }
                chi2n += wi * r * r;
            }
            /* predicted reduction: h^T (mu D^2 h + g) */
            double pred = 0.0;
            for (int j = 0; j < k; j++) pred += h[j] * (mu * dg[j] * dg[j] * h[j] + g[j]);
            double rho = (finite && pred > 0) ? (chi2 - chi2n) / pred : -1.0;
            if (rho > 0) {
                double actred = (chi2 - chi2n) / (chi2 > 0 ? chi2 : 1.0);
                double prered = pred / (chi2 > 0 ? chi2 : 1.0);
                memcpy(p, pn, sizeof(double) * k);
                memcpy(f, fn_new, sizeof(double) * n);
                memcpy(jac, jac_new, sizeof(double) * n * k);
                double t = 2.0 * rho - 1.0;
                mu *= fmax(1.0 / 3.0, 1.0 - t * t * t);
                nu = 2.0;
                chi2 = chi2n;
                if ((fabs(actred) <= ftol && prered <= ftol) || hnorm <= xtol * pnorm) {
                    status = 0;
                    it++;
                    goto done;
                }
                break;
            }
            mu *= nu; nu *= 2.0;
            if (hnorm <= xtol * pnorm || mu > 1e300) { status = 0; it++; goto done; }
        }
    }
done:
    if (status != 2) {
        /* final chi2 / weighted Jacobian at p */
        chi2 = 0.0;
        for (int i = 0; i < n; i++) {
            double wi = w ? w[i] : 1.0, r = y[i] - f[i];
            chi2 += wi * r * r;
            if (jw)
                for (int j = 0; j < k; j++) jw[(size_t)i * k + j] = sqrt(wi) * jac[(size_t)i * k + j];
        }
    }
    if (info) { info->chi2 = chi2; info->iters = it; info->evals = evals; }
    free(f);
    return status;
}

/* ------------------------------------------------------------------------ */
/* Bleach fits.                                                               */
/* ------------------------------------------------------------------------ */
/* PolynomFit (java:10953-11004): linear least squares of order `order` in t.
 * The LM of the Java code converges to the same linear least-squares
 * solution; it is computed directly here by Householder QR in the scaled
 * variable u = t / max|t| and converted back to powers of t. */
int imfcs_o_poly_fit(const double *y, const double *t, int n, int order, double *coef)
{
    int k = order + 1;
    double tmax = 0.0;
    for (int i = 0; i < n; i++) tmax = fmax(tmax, fabs(t[i]));
    if (tmax == 0.0 || n < k) return 1;
    double *a = (double *)malloc(sizeof(double) * n * (k + 1));
    double *b = a + (size_t)n * k;
    for (int i = 0; i < n; i++) {
        double u = t[i] / tmax, pw = 1.0;
        for (int j = 0; j < k; j++) { a[(size_t)i * k + j] = pw; pw *= u; }
        b[i] = y[i];
    }
    double rdiag[16];
    for (int c = 0; c < k; c++) {
        double nrm = 0.0;
        for (int r = c; r < n; r++) nrm += SQR(a[(size_t)r * k + c]);
        nrm = sqrt(nrm);
        double alpha = a[(size_t)c * k + c] > 0 ? -nrm : nrm;
        rdiag[c] = alpha;
        if (alpha == 0.0) { free(a); return 1; }
        a[(size_t)c * k + c] -= alpha;
        double vnorm = alpha * a[(size_t)c * k + c];   // = -v^T v / 2
        for (int cc = c + 1; cc <= k; cc++) {
            double dot = 0.0;
            if (cc < k) {
                for (int r = c; r < n; r++) dot += a[(size_t)r * k + c] * a[(size_t)r * k + cc];
                dot /= vnorm;
                for (int r = c; r < n; r++) a[(size_t)r * k + cc] += dot * a[(size_t)r * k + c];
            } else {
                for (int r = c; r < n; r++) dot += a[(size_t)r * k + c] * b[r];
                dot /= vnorm;
                for (int r = c; r < n; r++) b[r] += dot * a[(size_t)r * k + c];
            }
        }
    }
    double cu[16];
    for (int i = k - 1; i >= 0; i--) {
        double s = b[i];
        for (int j = i + 1; j < k; j++) s -= a[(size_t)i * k + j] * cu[j];
        cu[i] = s / rdiag[i];
    }
    double sc = 1.0;
    for (int j = 0; j < k; j++) { coef[j] = cu[j] / sc; sc *= tmax; }
    free(a);
    return 0;
}

typedef struct { const double *t; int n; int two; } expfit_ctx;

/* SingleExp / DoubleExp value and gradient (java:13028-13085). */
static void expfit_model(const double *p, double *f, double *jac, void *vctx)
{
    expfit_ctx *c = (expfit_ctx *)vctx;
    for (int i = 0; i < c->n; i++) {
        double x = c->t[i];
        if (!c->two) {
            double e = exp(-x / p[1]);
            f[i] = p[0] * e + p[2];
            jac[i * 3 + 0] = e;
            jac[i * 3 + 1] = p[0] * x * e / (p[1] * p[1]);
            jac[i * 3 + 2] = 1.0;
        } else {
            double e1 = exp(-x / p[1]), e2 = exp(-x / p[3]);
            f[i] = p[0] * e1 + p[2] * e2 + p[4];
            jac[i * 5 + 0] = e1;
            jac[i * 5 + 1] = p[0] * x * e1 / (p[1] * p[1]);
            jac[i * 5 + 2] = e2;
            jac[i * 5 + 3] = p[2] * x * e2 / (p[3] * p[3]);
            jac[i * 5 + 4] = 1.0;
        }
    }
}

/* u(k, t) = (1 - e^{-kt}) / k and its first two k-derivatives, stable for
 * any sign of k (series in x = kt for |x| < 0.05). */
static void exp_u3(double k, double t, double *u, double *uk, double *ukk)
{
    const double x = k * t;
    if (fabs(x) < 0.05) {
        /* u = t sum_m (-x)^m / (m+1)!,  u_k = -t^2 sum_m (m+1) (-x)^m / (m+2)!,
         * u_kk = t^3 sum_m (m+1)(m+2) (-x)^m / (m+3)! */
        double su = 0.0, sk = 0.0, skk = 0.0, p = 1.0, f1 = 1.0, f2 = 2.0, f3 = 6.0;
        for (int m = 0; m < 12; m++) {
            su += p / f1;
            sk += (m + 1) * p / f2;
            skk += (m + 1) * (m + 2) * p / f3;
            p *= -x;
            f1 *= (m + 2);
            f2 *= (m + 3);
            f3 *= (m + 4);
        }
        *u = t * su;
        *uk = -t * t * sk;
        *ukk = t * t * t * skk;
        return;
    }
    const double e = exp(-x);
    *u = (1.0 - e) / k;
    *uk = (t * e - *u) / k;
    *ukk = (-t * t * e - 2.0 * *uk) / k;
}

/* Exponential bleach fits in the rate form
 *     f(t) = f0 - sum_c s_c (1 - e^{-k_c t}) / k_c,   k_c >= 0
 * (s_c = A_c k_c, k_c = 1/tau_c, f0 = C + sum A_c): the same curves as the
 * reference's A e^{-t/tau} + C (java:13028-13085), continuous through k = 0
 * (tau = infinity, where A and C diverge with opposite signs; the linear
 * limit f0 - s t).  The reference's LM moves in A, tau, C and cannot cross
 * tau = infinity: on a trace whose least-squares minimum lies at or beyond
 * that valley it stops in the valley, on the k -> 0+ side, at a point set by
 * its stopping tolerances.  So the fit here is the least-squares minimum over
 * k >= 0: the reference's LM from its initial values, then a Newton polish
 * in the rate form with the full Hessian of chi^2/2, H = J^T J -
 * sum_i r_i d2f_i (the Gauss-Newton matrix alone does not contract on these
 * large-residual problems) and a rate held at 0 when its step points below
 * (active set), while chi^2 does not increase and H is positive definite,
 * until |h_j| <= 1e-12 (|p_j| + sigma_j).  The reference's commons-math LM
 * stops on relative cost / parameter tolerances of 1e-10, i.e. within about
 * 1e-4 standard errors of the minimum; where the bleach correction is
 * ill-conditioned (an averaged trace of a few photons in Java's int
 * division) that stopping point moves G by more than the parity tolerance,
 * so parity is defined on the minimum.  (Deviation from the Java stopping
 * point, stated here once.) */
static void exp_rate_polish(const double *t, const double *y, int n, int nc, double *p)
{
    const int k = 1 + 2 * nc;
    for (int it = 0; it < 60; it++) {
        double a[25] = {0}, g[5] = {0}, l[25], h[5], pn[5];
        double chi2 = 0.0;
        for (int i = 0; i < n; i++) {
            double f = p[0], jac[5], hs[5][5] = {{0}};
            jac[0] = 1.0;
            for (int c = 0; c < nc; c++) {
                double u, uk, ukk;
                exp_u3(p[2 + 2 * c], t[i], &u, &uk, &ukk);
                f -= p[1 + 2 * c] * u;
                jac[1 + 2 * c] = -u;
                jac[2 + 2 * c] = -p[1 + 2 * c] * uk;
                hs[1 + 2 * c][2 + 2 * c] = hs[2 + 2 * c][1 + 2 * c] = -uk;
                hs[2 + 2 * c][2 + 2 * c] = -p[1 + 2 * c] * ukk;
            }
            const double r = y[i] - f;
            chi2 += r * r;
            for (int j = 0; j < k; j++) {
                g[j] += jac[j] * r;
                for (int m = 0; m < k; m++) a[j * k + m] += jac[j] * jac[m] - r * hs[j][m];
            }
        }
        if (!isfinite(chi2)) return;
        int fix = 0;
        for (int pass = 0; pass < 2; pass++) {
            double aa[25], gg[5];
            memcpy(aa, a, sizeof(aa));
            memcpy(gg, g, sizeof(gg));
            for (int j = 0; j < k; j++)
                if ((fix >> j) & 1) {
                    for (int m = 0; m < k; m++) aa[j * k + m] = aa[m * k + j] = 0.0;
                    aa[j * k + j] = 1.0;
                    gg[j] = 0.0;
                }
            memcpy(l, aa, sizeof(double) * k * k);
            if (chol_inplace(l, k)) return;     /* not in the convex region */
            chol_solve(l, k, gg, h);
            int more = 0;
            for (int c = 0; c < nc; c++) {
                const int jk = 2 + 2 * c;
                if (!((fix >> jk) & 1) && p[jk] <= 0.0 && h[jk] < 0.0) { fix |= 1 << jk; more = 1; }
            }
            if (!more) break;
        }
        int small = 1;
        for (int j = 0; j < k; j++) {
            double e[5], col[5];
            for (int m = 0; m < k; m++) e[m] = (m == j);
            chol_solve(l, k, e, col);
            const double sig = sqrt(fabs(col[j]) * chi2 / (n > k ? n - k : 1));
            if (!(fabs(h[j]) <= 1e-12 * (fabs(p[j]) + sig))) small = 0;
            pn[j] = p[j] + h[j];
        }
        for (int c = 0; c < nc; c++) pn[2 + 2 * c] = fmax(pn[2 + 2 * c], 0.0);
        double chi2n = 0.0;
        for (int i = 0; i < n; i++) {
            double f = pn[0];
            for (int c = 0; c < nc; c++) {
                double u, uk, ukk;
                exp_u3(pn[2 + 2 * c], t[i], &u, &uk, &ukk);
                f -= pn[1 + 2 * c] * u;
            }
            chi2n += SQR(y[i] - f);
        }
        if (!(isfinite(chi2n) && chi2n <= chi2)) return;
        memcpy(p, pn, sizeof(double) * k);
        if (small) return;
    }
}

/* Global search for the single-exponential fit by variable projection: for a
 * rate k the curve c0 + c1 e^{-kt} (k = 0: c0 + c1 t, the linear limit) is
 * linear in c0, c1, so chi^2(k) is minimised over them exactly; k runs over
 * a fixed grid, x = k tmax in {0} and 96 log-spaced values 1e-3 .. 1e4
 * (tmax = the last averaged point's time), the best grid rate is refined by
 * golden section between its neighbours.  The GPU path scans the same grid.
 * Returns chi^2 at k and the linear parameters. */
#define EXP_GRID 97
static double exp_grid_x(int j) { return j == 0 ? 0.0 : pow(10.0, -3.0 + 7.0 * (j - 1) / 95.0); }

static double varpro_chi2(const double *t, const double *y, int n, double k, double *c0, double *c1)
{
    double sy = 0.0, se = 0.0;
    for (int i = 0; i < n; i++) {
        sy += y[i];
        se += k == 0.0 ? t[i] : exp(-k * t[i]);
    }
    const double my = sy / n, me = se / n;
    double see = 0.0, sye = 0.0, syy = 0.0;
    for (int i = 0; i < n; i++) {
        const double e = (k == 0.0 ? t[i] : exp(-k * t[i])) - me, yc = y[i] - my;
        see += e * e;
        sye += yc * e;
        syy += yc * yc;
    }
    *c1 = see > 0.0 ? sye / see : 0.0;
    *c0 = my - *c1 * me;
    return syy - *c1 * sye;
}

/* Rate form (f0, s, k) of the global single-exponential minimum over k >= 0. */
static void exp_fit_global(const double *t, const double *y, int n, double *rate)
{
    const double tmax = t[n - 1];
    int best = 0;
    double bc = INFINITY, c0, c1;
    for (int j = 0; j < EXP_GRID; j++) {
        const double c = varpro_chi2(t, y, n, exp_grid_x(j) / tmax, &c0, &c1);
        if (c < bc) { bc = c; best = j; }
    }
    /* golden section on x between the neighbours of the best grid point */
    double a = best > 0 ? exp_grid_x(best - 1) : 0.0;
    double b = best < EXP_GRID - 1 ? exp_grid_x(best + 1) : exp_grid_x(best);
    const double gr = 0.5 * (sqrt(5.0) - 1.0);
    double x1 = b - gr * (b - a), x2 = a + gr * (b - a);
    double f1 = varpro_chi2(t, y, n, x1 / tmax, &c0, &c1), f2 = varpro_chi2(t, y, n, x2 / tmax, &c0, &c1);
    for (int it = 0; it < 200 && b - a > 1e-14 * (fabs(a) + fabs(b)) + 1e-300; it++) {
        if (f1 <= f2) { b = x2; x2 = x1; f2 = f1; x1 = b - gr * (b - a); f1 = varpro_chi2(t, y, n, x1 / tmax, &c0, &c1); }
        else { a = x1; x1 = x2; f1 = f2; x2 = a + gr * (b - a); f2 = varpro_chi2(t, y, n, x2 / tmax, &c0, &c1); }
    }
    double x = 0.5 * (a + b);
    if (varpro_chi2(t, y, n, 0.0, &c0, &c1) <= varpro_chi2(t, y, n, x / tmax, &c0, &c1)) x = 0.0;
    const double k = x / tmax;
    varpro_chi2(t, y, n, k, &c0, &c1);
    if (k == 0.0) { rate[0] = c0; rate[1] = -c1; rate[2] = 0.0; }      /* f = c0 + c1 t */
    else { rate[0] = c0 + c1; rate[1] = c1 * k; rate[2] = k; }           /* f = c0 + c1 e^{-kt} */
}

/* rate[] = f0, s1, k1 [, s2, k2].  Single exponential: the global minimum
 * over k >= 0 (variable projection on the rate grid), polished.  Double
 * exponential: the reference's LM from its initial values (java:10917-10921)
 * and the rate-form polish.  Returns 0 on success. */
static int exp_fit_rate(const double *y, const double *t, int n, int two, double *rate)
{
    if (!two) {
        exp_fit_global(t, y, n, rate);
        exp_rate_polish(t, y, n, 1, rate);
        return (isfinite(rate[0]) && isfinite(rate[1]) && isfinite(rate[2])) ? 0 : 1;
    }
    expfit_ctx c = {t, n, two};
    double res[5];
    if (!two) {
        res[0] = y[1];
        res[1] = t[n / 2];
        res[2] = 0.0;
    } else {
        res[0] = y[1] / 2;
        res[1] = t[n / 10];
        res[2] = y[1] / 2;
        res[3] = t[n / 2];
        res[4] = 0.0;
    }
    lm_info info;
    const int nc = two ? 2 : 1;
    if (lm_solve(expfit_model, &c, n, 1 + 2 * nc, y, NULL, res, 100000, &info, NULL) == 2) return 1;
    double f0 = res[two ? 4 : 2];
    for (int m = 0; m < nc; m++) {
        const double A = res[2 * m], tau = res[2 * m + 1];
        if (!(isfinite(A) && isfinite(tau)) || tau == 0.0) return 1;
        rate[1 + 2 * m] = A / tau;                 /* s = A k */
        rate[2 + 2 * m] = fmax(1.0 / tau, 0.0);    /* k >= 0 */
        f0 += A;
    }
    rate[0] = f0;
    exp_rate_polish(t, y, n, nc, rate);
    return 0;
}

/* rate form -> A, tau, C (tau = +inf, A = +-inf, C = -A for k = 0) */
static void rate_to_reference(const double *rate, int nc, double *res)
{
    double C = rate[0];
    for (int m = 0; m < nc; m++) {
        const double s = rate[1 + 2 * m], k = rate[2 + 2 * m];
        res[2 * m] = k > 0.0 ? s / k : copysign(INFINITY, s);
        res[2 * m + 1] = k > 0.0 ? 1.0 / k : INFINITY;
        C -= res[2 * m];
    }
    res[2 * nc] = C;
}

/* The rate-form fit (f0, s1, k1 [, s2, k2]) and the standard errors of its
 * parameters, sqrt(diag((J^T J)^-1) chi2 / (n - k)) at the solution: a rate
 * whose standard error is at least its value is not determined by the trace
 * (a decay faster than the first averaged point, fitted to one non-zero
 * point, or a curve in the tau -> infinity valley), so where an optimiser
 * stops on it is arbitrary.  Returns 0 on success. */
int imfcs_o_exp_fit_rate(const double *y, const double *t, int n, int two, double *rate, double *sigma)
{
    if (exp_fit_rate(y, t, n, two, rate)) return 1;
    const int nc = two ? 2 : 1, k = 1 + 2 * nc;
    double a[25] = {0}, l[25], chi2 = 0.0;
    for (int i = 0; i < n; i++) {
        double f = rate[0], jac[5];
        jac[0] = 1.0;
        for (int c = 0; c < nc; c++) {
            double u, uk, ukk;
            exp_u3(rate[2 + 2 * c], t[i], &u, &uk, &ukk);
            f -= rate[1 + 2 * c] * u;
            jac[1 + 2 * c] = -u;
            jac[2 + 2 * c] = -rate[1 + 2 * c] * uk;
        }
        chi2 += SQR(y[i] - f);
        for (int j = 0; j < k; j++)
            for (int m = 0; m < k; m++) a[j * k + m] += jac[j] * jac[m];
    }
    memcpy(l, a, sizeof(l));
    if (chol_inplace(l, k)) {
        for (int j = 0; j < k; j++) sigma[j] = INFINITY;
        return 0;
    }
    for (int j = 0; j < k; j++) {
        double e[5], col[5];
        for (int m = 0; m < k; m++) e[m] = (m == j);
        chol_solve(l, k, e, col);
        sigma[j] = sqrt(fabs(col[j]) * chi2 / (n > k ? n - k : 1));
    }
    return 0;
}

int imfcs_o_exp_fit(const double *y, const double *t, int n, double *res3)
{
    double rate[3];
    if (exp_fit_rate(y, t, n, 0, rate)) return 1;
    rate_to_reference(rate, 1, res3);
    return 0;
}

int imfcs_o_dexp_fit(const double *y, const double *t, int n, double *res5)
{
    double rate[5];
    if (exp_fit_rate(y, t, n, 1, rate)) return 1;
    rate_to_reference(rate, 2, res5);
    return 0;
}

/* The exponential correction (java:9689-9692, 9714-9717) from rate-form
 * parameters: f(t)/f0 with the curve continuous through k = 0.  The
 * reference skips the correction when A tau (A1 tau1 A2 tau2) is 0, i.e.
 * when a slope s is 0. */
static void bleach_apply_rate(double *intdat, int num, double frametime, int nc, const double *rate)
{
    const double f0 = rate[0];
    for (int m = 0; m < nc; m++)
        if (rate[1 + 2 * m] == 0.0) return;
    for (int x = 1; x <= num; x++) {
        const double tt = frametime * (x + 0.5);
        double f = f0;
        for (int m = 0; m < nc; m++) {
            double u, uk, ukk;
            exp_u3(rate[2 + 2 * m], tt, &u, &uk, &ukk);
            f -= rate[1 + 2 * m] * u;
        }
        const double r = f / f0;
        intdat[x] = intdat[x] / sqrt(r) + f0 * (1 - sqrt(r));
    }
}

void imfcs_o_bleach_apply(double *intdat, int num, double frametime, int mode, int order,
                          const double *res)
{
    if (mode == IMFCS_O_BLEACH_SINGLE_EXP) {       /* java:9689-9692 */
        if (res[0] * res[1] == 0) return;
        for (int x = 1; x <= num; x++) {
            double f = (res[0] * exp(-frametime * (x + 0.5) / res[1]) + res[2]) / (res[0] + res[2]);
            intdat[x] = intdat[x] / sqrt(f) + (res[0] + res[2]) * (1 - sqrt(f));
        }
    } else if (mode == IMFCS_O_BLEACH_DOUBLE_EXP) { /* java:9714-9717 */
        if (res[0] * res[1] * res[2] * res[3] == 0) return;
        for (int x = 1; x <= num; x++) {
            double tt = frametime * (x + 0.5);
            double f0 = res[0] + res[2] + res[4];
            double f = (res[0] * exp(-tt / res[1]) + res[2] * exp(-tt / res[3]) + res[4]) / f0;
            intdat[x] = intdat[x] / sqrt(f) + f0 * (1 - sqrt(f));
        }
    } else if (mode == IMFCS_O_BLEACH_POLY) {      /* java:9744-9750 */
        for (int x = 1; x <= num; x++) {
            double corfunc = 0.0;
            for (int i = 0; i <= order; i++) corfunc += res[i] * pow(frametime * (x + 0.5), i);
            intdat[x] = intdat[x] / sqrt(corfunc / res[0]) + res[0] * (1 - sqrt(corfunc / res[0]));
        }
    }
}

/* ------------------------------------------------------------------------ */
/* blockTransform (java:9217-9422).                                          */
/* ------------------------------------------------------------------------ */
int imfcs_o_block_transform(const double *c0, const double *c1, int num, int p, int q,
                            const int *lag, const double *samp, const double *mtab,
                            double frametime, int *block_ind_s, double *varblock)
{
    const int blocklag = 1;
    int chanum = imfcs_o_chanum(p, q);
    int blocknum = (int)floor(log(mtab[blocklag]) / log(2)) - 2;
    int numbin = num, ind = 0, last0 = 0;
    double sumprod = 0.0, sumprod2 = 0.0, directm = 0.0, delayedm = 0.0;
    double *ib0 = (double *)malloc(sizeof(double) * (3 * (size_t)num + 8 * (size_t)blocknum + 8));
    double *ib1 = ib0 + num, *prod = ib1 + num;
    double *vb0 = prod + num, *vb1 = vb0 + blocknum, *vb2 = vb1 + blocknum;
    double *upper = vb2 + blocknum, *lower = upper + blocknum, *prodnum = lower + blocknum;
    int crt[64] = {0}, cr12[64] = {0}, cr3[64] = {0}, diffpos[64] = {0};

    for (int x = 0; x < numbin; x++) { ib0[x] = c0[x]; ib1[x] = c1[x]; }
    int cur = blocklag;
    for (int x = 1; x < chanum; x++) {
        if (cur != samp[x]) {
            cur = (int)samp[x];
            numbin = (int)floor(numbin / 2);
            for (int y = 0; y < numbin; y++) {
                ib0[y] = ib0[2 * y] + ib0[2 * y + 1];
                ib1[y] = ib1[2 * y] + ib1[2 * y + 1];
            }
        }
        if (x == blocklag) {
            int del = lag[x] / cur;
            for (int y = 0; y < numbin - del; y++) { directm += ib0[y]; delayedm += ib1[y + del]; }
            prodnum[0] = numbin - del;
            directm /= prodnum[0];
            delayedm /= prodnum[0];
            for (int y = 0; y < prodnum[0]; y++) {
                prod[y] = ib0[y] * ib1[y + del] - delayedm * ib0[y] - directm * ib1[y + del] +
                          delayedm * directm;
                sumprod += prod[y];
                sumprod2 += prod[y] * prod[y];
            }
            vb0[0] = cur * frametime;
            vb1[0] = (sumprod2 / prodnum[0] - SQR(sumprod / prodnum[0])) /
                     (prodnum[0] * SQR(directm * delayedm));
            for (int y = 1; y < blocknum; y++) {
                prodnum[y] = (int)floor(prodnum[y - 1] / 2);
                sumprod = 0; sumprod2 = 0;
                for (int z = 0; z < prodnum[y]; z++) {
                    prod[z] = (prod[2 * z] + prod[2 * z + 1]) / 2;
                    sumprod += prod[z];
                    sumprod2 += prod[z] * prod[z];
                }
                vb0[y] = (cur * pow(2, y)) * frametime;
                vb1[y] = (sumprod2 / prodnum[y] - SQR(sumprod / prodnum[y])) /
                         (prodnum[y] * SQR(directm * delayedm));
            }
        }
    }
    for (int x = 0; x < blocknum; x++) {
        vb1[x] = sqrt(vb1[x]);
        vb2[x] = vb1[x] / sqrt(2 * (prodnum[x] - 1));
        upper[x] = vb1[x] + vb2[x];
        lower[x] = vb1[x] - vb2[x];
    }
    for (int x = 0; x < blocknum - 1; x++)
        if (upper[x] > lower[x + 1] && upper[x + 1] > lower[x]) crt[x] = 1;
    for (int x = 0; x < blocknum - 2; x++)
        if (crt[x] * crt[x + 1] == 1) cr12[x] = 1;
    for (int x = 0; x < blocknum - 1; x++)
        if (vb1[x + 1] - vb1[x] > 0) diffpos[x] = 1;
    for (int x = 0; x < blocknum - 2; x++)
        if (diffpos[x] * diffpos[x + 1] == 1) cr3[x] = 1;
    for (int x = 0; x < blocknum - 2; x++)
        if (cr3[x] == 1 && cr12[x] == 0) last0 = x;
    for (int x = 0; x <= last0; x++) cr12[x] = 0;
    cr12[blocknum - 3] = 0;
    cr12[blocknum - 4] = 0;
    for (int x = blocknum - 5; x > 0; x--)
        if (cr12[x] == 1) ind = x + 1;
    if (ind == 0) {
        *block_ind_s = 0;
        ind = (blocknum - 3 > 0) ? blocknum - 3 : blocknum - 1;
    } else {
        *block_ind_s = 1;
    }
    if (ind < q - 1) ind = q - 1;
    if (varblock)
        for (int x = 0; x < blocknum; x++) {
            varblock[x] = vb0[x];
            varblock[blocknum + x] = vb1[x];
            varblock[2 * blocknum + x] = vb2[x];
        }
    free(ib0);
    return ind;
}

/* ------------------------------------------------------------------------ */
/* calculateCF (java:9425-9648).                                             */
/* ------------------------------------------------------------------------ */
void imfcs_o_calculate_cf(const double *c0, const double *c1, int num, int ind, int p, int q,
                          const int *lag, const double *samp, const double *mtab, int gls,
                          double *corav, double *blockvar, double *blocksd, double *covmats)
{
    int chanum = imfcs_o_chanum(p, q);
    int numbin = num, ctbin = 0;
    int pnum = (int)floor(mtab[chanum - 1] /
                          pow(2, fmax(ind - log(samp[chanum - 1]) / log(2), 0)));
    double *ib0 = (double *)malloc(sizeof(double) * (3 * (size_t)num));
    double *ib1 = ib0 + num, *prod = ib1 + num;
    double *bprod = (double *)malloc(sizeof(double) * (size_t)chanum * (pnum > 0 ? pnum : 1));
    double *dm = (double *)calloc(chanum, sizeof(double));
    double *Dm = (double *)calloc(chanum, sizeof(double));

    for (int x = 0; x < numbin; x++) { ib0[x] = c0[x + 1]; ib1[x] = c1[x + 1]; }
    int cur = 1;
    for (int x = 0; x < chanum; x++) {
        if (cur != samp[x]) {
            numbin = (int)floor(numbin / 2);
            cur = (int)samp[x];
            ctbin++;
            for (int y = 0; y < numbin; y++) {
                ib0[y] = ib0[2 * y] + ib0[2 * y + 1];
                ib1[y] = ib1[2 * y] + ib1[2 * y + 1];
            }
        }
        int del = lag[x] / cur;
        int prodnum = numbin - del;
        for (int y = 0; y < prodnum; y++) { dm[x] += ib0[y]; Dm[x] += ib1[y + del]; }
        dm[x] /= prodnum;
        Dm[x] /= prodnum;
        double sumprod = 0.0, sumprod2 = 0.0;
        for (int y = 0; y < prodnum; y++) {
            prod[y] = ib0[y] * ib1[y + del] - Dm[x] * ib0[y] - dm[x] * ib1[y + del] + Dm[x] * dm[x];
            sumprod += prod[y];
            sumprod2 += prod[y] * prod[y];
        }
        corav[x] = sumprod / (prodnum * dm[x] * Dm[x]);
        int binct = ind - ctbin;
        for (int y = 1; y <= binct; y++) {
            prodnum = (int)floor(prodnum / 2);
            for (int z = 0; z < prodnum; z++) prod[z] = (prod[2 * z] + prod[2 * z + 1]) / 2;
        }
        sumprod = 0.0; sumprod2 = 0.0;
        for (int z = 0; z < pnum; z++) {
            sumprod += prod[z];
            sumprod2 += prod[z] * prod[z];
            bprod[(size_t)x * pnum + z] = prod[z];
        }
        blockvar[x] = (sumprod2 / pnum - SQR(sumprod / pnum)) / ((pnum - 1) * SQR(dm[x] * Dm[x]));
        blocksd[x] = sqrt(blockvar[x]);
    }

    if (gls) {
        int n1 = chanum - 1;
        double *mcov = (double *)calloc(chanum, sizeof(double));
        double *cov = (double *)calloc((size_t)chanum * chanum, sizeof(double));
        double *cor = (double *)calloc((size_t)chanum * chanum, sizeof(double));
        double *diag = (double *)calloc(chanum, sizeof(double));
        double numerator = 0.0, denominator = 0.0, median, tmpnum, lamvar, lamcov;
#define BP(x, z) (bprod[(size_t)(x) * pnum + (z)] / (dm[x] * Dm[x]))
        for (int x = 1; x < chanum; x++) {
            for (int z = 0; z < pnum; z++) mcov[x] += BP(x, z);
            mcov[x] /= pnum;
        }
        for (int x = 1; x < chanum; x++)
            for (int y = 1; y <= x; y++) {
                double s = 0.0;
                for (int z = 0; z < pnum; z++) s += (BP(x, z) - mcov[x]) * (BP(y, z) - mcov[y]);
                s /= (pnum - 1);
                cov[x * chanum + y] = s;
                cov[y * chanum + x] = s;
            }
        /* median over chanum entries incl. the unset zero-lag slot (java:9563-9573) */
        for (int x = 1; x < chanum; x++) diag[x] = cov[x * chanum + x];
        for (int i = 1; i < chanum; i++) { /* insertion sort */
            double v = diag[i];
            int j = i - 1;
            while (j >= 0 && diag[j] > v) { diag[j + 1] = diag[j]; j--; }
            diag[j + 1] = v;
        }
        {
            double pos1 = floor((chanum - 1.0) / 2.0), pos2 = ceil((chanum - 1.0) / 2.0);
            median = (pos1 == pos2) ? diag[(int)pos1] : (diag[(int)pos1] + diag[(int)pos2]) / 2.0;
        }
        for (int x = 1; x < chanum; x++) {
            tmpnum = 0.0;
            for (int z = 0; z < pnum; z++)
                tmpnum += SQR(SQR(BP(x, z) - mcov[x]) - cov[x * chanum + x]);
            tmpnum *= pnum / pow(pnum - 1, 3);
            numerator += tmpnum;
            denominator += SQR(cov[x * chanum + x] - median);
        }
        lamvar = fmin(1, numerator / denominator);
        lamvar = fmax(lamvar, 0);
        for (int x = 1; x < chanum; x++)
            for (int y = 1; y < chanum; y++)
                cor[x * chanum + y] = cov[x * chanum + y] / sqrt(cov[x * chanum + x] * cov[y * chanum + y]);
        numerator = 0.0; denominator = 0.0;
        for (int x = 1; x < chanum; x++) {
            tmpnum = 0.0; /* not reset per y, and rescaled inside the y loop (java:9592-9603) */
            for (int y = 1; y < x; y++) {
                for (int z = 0; z < pnum; z++) {
                    double cmx = (BP(x, z) - mcov[x]) / sqrt(cov[x * chanum + x]);
                    double cmy = (BP(y, z) - mcov[y]) / sqrt(cov[y * chanum + y]);
                    tmpnum += SQR(cmx * cmy - cor[x * chanum + y]);
                }
                tmpnum *= pnum / pow(pnum - 1, 3);
                numerator += tmpnum;
                denominator += SQR(cor[x * chanum + y]);
            }
        }
        lamcov = fmin(1, numerator / denominator);
        lamcov = fmax(lamcov, 0);
        for (int x = 1; x < chanum; x++)
            for (int y = 1; y < x; y++) {
                double cmx = lamvar * median + (1 - lamvar) * cov[x * chanum + x];
                double cmy = lamvar * median + (1 - lamvar) * cov[y * chanum + y];
                double v = (1 - lamcov) * cor[x * chanum + y] * sqrt(cmx * cmy) / pnum;
                covmats[(size_t)(x - 1) * n1 + (y - 1)] = v;
                covmats[(size_t)(y - 1) * n1 + (x - 1)] = v;
            }
        for (int x = 1; x < chanum; x++)
            covmats[(size_t)(x - 1) * n1 + (x - 1)] =
                (lamvar * median + (1 - lamvar) * cov[x * chanum + x]) / pnum;
        for (int x = 0; x < chanum; x++) corav[x] = mcov[x]; /* java:9638-9642 */
#undef BP
        free(mcov); free(cov); free(cor); free(diag);
    }
    free(ib0); free(bprod); free(dm); free(Dm);
}

/* ------------------------------------------------------------------------ */
/* FCS_3p model (java:13131-13408).  par: N, D, vx, vy, G, F2, D2, F3, D3,   */
/* Ftrip, Ttrip (SI units).  cst: ax, ay, s, sz, rx, ry, fitobsvol, q2, q3.  */
/* The gradient is derived independently (d/dp0 of the lateral term is       */
/* (e1 + e2 - 2 e3)/sqrt(pi), d/dp of p*erf(p/p0)+p0/sqrt(pi)*e is erf).     */
/* ------------------------------------------------------------------------ */
static const double O_PI = 3.14159265359; /* the Java constant (java:13134) */

typedef struct { double lat, dlat_dd, dlat_dvx, dlat_dvy, psp, dpsp_dd; } comp_terms;

static void lateral_1d(double a, double r, double v, double tau, double p0, double *L,
                       double *dL_dp0, double *dL_dv)
{
    double sqrpi = sqrt(O_PI);
    double p1 = a + r - v * tau, p2 = a - r + v * tau, p3 = r - v * tau;
    double u1 = p1 / p0, u2 = p2 / p0, u3 = p3 / p0;
    double e1 = exp(-u1 * u1), e2 = exp(-u2 * u2), e3 = exp(-u3 * u3);
    double er1 = erf(u1), er2 = erf(u2), er3 = erf(u3);
    *L = p0 / sqrpi * (e1 + e2 - 2 * e3) + p1 * er1 + p2 * er2 - 2 * p3 * er3;
    *dL_dp0 = (e1 + e2 - 2 * e3) / sqrpi;
    *dL_dv = (er2 + 2 * er3 - er1) * tau;
}

static void component(double d, const double *par, const double *cst, double tau,
                      comp_terms *o)
{
    double ax = cst[0], ay = cst[1], s = cst[2], sz = cst[3], rx = cst[4], ry = cst[5];
    double norm = 4 * SQR(ax * ay) / cst[6];
    double p0 = sqrt(4 * d * tau + s * s);
    double Lx, Ly, dLx0, dLy0, dLxv, dLyv;
    lateral_1d(ax, rx, par[2], tau, p0, &Lx, &dLx0, &dLxv);
    lateral_1d(ay, ry, par[3], tau, p0, &Ly, &dLy0, &dLyv);
    double dp0 = 2 * tau / p0;
    o->lat = Lx * Ly / norm;
    o->dlat_dd = (dLx0 * dp0 * Ly + Lx * dLy0 * dp0) / norm;
    o->dlat_dvx = dLxv * Ly / norm;
    o->dlat_dvy = Lx * dLyv / norm;
    double q = 1 + 4 * d * tau / (sz * sz);
    o->psp = 1 / sqrt(q);
    o->dpsp_dd = -2 * tau / (sz * sz) * o->psp * o->psp * o->psp;
}

void imfcs_o_fcs_model(const double *par, const double *cst, double tau, double *value,
                       double *grad)
{
    double N = par[0], F2 = par[5], F3 = par[7], Ft = par[9], Tt = par[10];
    double q2 = cst[7], q3 = cst[8];
    comp_terms c1, c2, c3;
    component(par[1], par, cst, tau, &c1);
    component(par[6], par, cst, tau, &c2);
    component(par[8], par, cst, tau, &c3);
    double a1 = c1.lat * c1.psp, a2 = c2.lat * c2.psp, a3 = c3.lat * c3.psp;
    double et = (Tt != 0.0) ? exp(-tau / Tt) : 0.0;
    double trip = 1 + Ft / (1 - Ft) * et;
    double Z = 1 - F2 - F3 + q2 * F2 + q3 * F3;
    double S = (1 - F2 - F3) * a1 + q2 * q2 * F2 * a2 + q3 * q3 * F3 * a3;
    double base = S / (Z * Z);
    *value = base / N * trip + par[4];
    if (!grad) return;
    double k = trip / (N * Z * Z);
    grad[0] = -base * trip / (N * N);
    grad[1] = k * (1 - F2 - F3) * (c1.dlat_dd * c1.psp + c1.lat * c1.dpsp_dd);
    grad[2] = k * ((1 - F2 - F3) * c1.dlat_dvx * c1.psp + q2 * q2 * F2 * c2.dlat_dvx * c2.psp +
                   q3 * q3 * F3 * c3.dlat_dvx * c3.psp);
    grad[3] = k * ((1 - F2 - F3) * c1.dlat_dvy * c1.psp + q2 * q2 * F2 * c2.dlat_dvy * c2.psp +
                   q3 * q3 * F3 * c3.dlat_dvy * c3.psp);
    grad[4] = 1.0;
    grad[5] = trip / N * ((-a1 + q2 * q2 * a2) / (Z * Z) - 2 * S * (q2 - 1) / (Z * Z * Z));
    grad[6] = k * q2 * q2 * F2 * (c2.dlat_dd * c2.psp + c2.lat * c2.dpsp_dd);
    grad[7] = trip / N * ((-a1 + q3 * q3 * a3) / (Z * Z) - 2 * S * (q3 - 1) / (Z * Z * Z));
    grad[8] = k * q3 * q3 * F3 * (c3.dlat_dd * c3.psp + c3.lat * c3.dpsp_dd);
    grad[9] = base / N * et / ((1 - Ft) * (1 - Ft));
    grad[10] = (Tt != 0.0) ? base / N * Ft / (1 - Ft) * et * tau / (Tt * Tt) : 0.0;
}

double imfcs_o_obsvol(double ax, double ay, double s)
{
    double sqrpi = sqrt(O_PI);
    double pexpx0 = 2 * exp(-SQR(ax / s)) - 2, perfx0 = 2 * ax * erf(ax / s);
    double pexpy0 = 2 * exp(-SQR(ay / s)) - 2, perfy0 = 2 * ay * erf(ay / s);
    return 4 * SQR(ax * ay) / ((s / sqrpi * pexpx0 + perfx0) * (s / sqrpi * pexpy0 + perfy0));
}

/* ------------------------------------------------------------------------ */
/* Fits.                                                                      */
/* ------------------------------------------------------------------------ */
/* Unit of each parameter in the LM's internal scaling (the Java UI units,
 * java:7464-7474): N, D [um^2/s], v [um/s], G, F2, D2, F3, D3, Ftrip, Ttrip [us]. */
static const double O_UNIT[IMFCS_O_NPARAM] = {1, 1e-12, 1e-6, 1e-6, 1, 1, 1e-12, 1, 1e-12, 1, 1e-6};

typedef struct {
    const double *lagtime; int n;      /* points: lagtime[0..n-1] */
    const double *init; const int *free_mask; const double *cst;
    int idx[IMFCS_O_NPARAM]; int k;
    const double *linv;                /* GLS: inverse-free forward-substitution L (n x n) */
    double *tmp;
} fcs_ctx;

static void fcs_expand(const fcs_ctx *c, const double *p, double *par)
{
    for (int i = 0; i < IMFCS_O_NPARAM; i++) par[i] = c->init[i];
    for (int j = 0; j < c->k; j++) par[c->idx[j]] = p[j] * O_UNIT[c->idx[j]];
}

static void fcs_points(const double *p, double *f, double *jac, void *vctx)
{
    fcs_ctx *c = (fcs_ctx *)vctx;
    double par[IMFCS_O_NPARAM], g[IMFCS_O_NPARAM];
    fcs_expand(c, p, par);
    for (int i = 0; i < c->n; i++) {
        imfcs_o_fcs_model(par, c->cst, c->lagtime[i], &f[i], g);
        for (int j = 0; j < c->k; j++) jac[(size_t)i * c->k + j] = g[c->idx[j]] * O_UNIT[c->idx[j]];
    }
    if (c->linv) { /* GLS: transform model and Jacobian by L^-1 (forward substitution) */
        int n = c->n, k = c->k;
        const double *L = c->linv;
        for (int i = 0; i < n; i++) {
            double s = f[i];
            for (int m = 0; m < i; m++) s -= L[(size_t)i * n + m] * f[m];
            f[i] = s / L[(size_t)i * n + i];
            for (int j = 0; j < k; j++) {
                double sj = jac[(size_t)i * k + j];
                for (int m = 0; m < i; m++) sj -= L[(size_t)i * n + m] * jac[(size_t)m * k + j];
                jac[(size_t)i * k + j] = sj / L[(size_t)i * n + i];
            }
        }
    }
}

/* Parameter covariance of the weighted problem in SI units with the
 * commons-math singularity threshold 1 (java:10412).  jw: n x k internal. */
static int param_cov(const double *jw, int n, int k, const int *idx, double *cov, double *sigma)
{
    double jtj[64 * 64], inv[64 * 64];
    if (k < 1 || k > 64) return 1;
    for (int a = 0; a < k; a++)
        for (int b = 0; b < k; b++) {
            double s = 0.0;
            for (int i = 0; i < n; i++) s += jw[(size_t)i * k + a] * jw[(size_t)i * k + b];
            jtj[a * k + b] = s / (O_UNIT[idx[a]] * O_UNIT[idx[b]]);
        }
    if (qr_inverse(jtj, k, 1.0, inv)) return 1;
    for (int a = 0; a < k * k; a++) if (cov) cov[a] = inv[a];
    for (int a = 0; a < k; a++) if (sigma) sigma[a] = sqrt(inv[a * k + a]);
    return 0;
}

int imfcs_o_fit_ols(const double *acf, const double *var, const double *lagtime, int chanum,
                    int fitstart, int fitend, const double *init, const int *free_mask,
                    const double *cst, int max_iter, double *out, double *chi2, double *cov,
                    double *sigma, double *tres, int *iters)
{
    fcs_ctx c;
    memset(&c, 0, sizeof(c));
    int n = fitend - fitstart + 1;
    c.lagtime = lagtime + fitstart; c.n = n; c.init = init; c.free_mask = free_mask; c.cst = cst;
    for (int i = 0; i < IMFCS_O_NPARAM; i++) if (free_mask[i]) c.idx[c.k++] = i;
    double p[IMFCS_O_NPARAM], w[512], jw[512 * IMFCS_O_NPARAM];
    for (int j = 0; j < c.k; j++) p[j] = init[c.idx[j]] / O_UNIT[c.idx[j]];
    for (int i = 0; i < n; i++) w[i] = 1.0 / var[fitstart + i];
    lm_info info;
    int st = lm_solve(fcs_points, &c, n, c.k, acf + fitstart, w, p, max_iter, &info, jw);
    if (iters) *iters = info.iters;
    if (st != 0) { for (int i = 0; i < IMFCS_O_NPARAM; i++) out[i] = NAN; return 1; }
    if (param_cov(jw, n, c.k, c.idx, cov, sigma)) {
        for (int i = 0; i < IMFCS_O_NPARAM; i++) out[i] = NAN;
        return 1;
    }
    fcs_expand(&c, p, out);
    /* reduced chi2 of the weighted residuals (java:10403-10406) */
    double x2 = 0.0;
    for (int i = fitstart; i <= fitend; i++) {
        double v; imfcs_o_fcs_model(out, cst, lagtime[i], &v, NULL);
        x2 += SQR(acf[i] - v) / var[i] / ((fitend - fitstart) - c.k - 1);
    }
    *chi2 = x2;
    if (tres)
        for (int i = 1; i < chanum; i++) {
            if (i >= fitstart && i <= fitend) {
                double v; imfcs_o_fcs_model(out, cst, lagtime[i], &v, NULL);
                tres[i - 1] = acf[i] - v;
            } else tres[i - 1] = 0.0;
        }
    return 0;
}

/* commons-math CholeskyDecomposition with its default thresholds
 * (relative symmetry 1e-15, absolute positivity 1e-10), java:13717. */
static int cm_cholesky(const double *m, int n, double *L)
{
    double *lt = (double *)malloc(sizeof(double) * n * n);
    memcpy(lt, m, sizeof(double) * n * n);
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double lij = lt[i * n + j], lji = lt[j * n + i];
            double md = 1e-15 * fmax(fabs(lij), fabs(lji));
            if (fabs(lij - lji) > md) { free(lt); return 1; }
            lt[j * n + i] = 0;
        }
    for (int i = 0; i < n; i++) {
        double *lti = lt + (size_t)i * n;
        if (lti[i] <= 1e-10) { free(lt); return 2; }
        lti[i] = sqrt(lti[i]);
        double inverse = 1.0 / lti[i];
        for (int qq = n - 1; qq > i; qq--) {
            lti[qq] *= inverse;
            double *ltq = lt + (size_t)qq * n;
            for (int pp = qq; pp < n; pp++) ltq[pp] -= lti[qq] * lti[pp];
        }
    }
    /* L = lt^T */
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) L[(size_t)i * n + j] = (j <= i) ? lt[(size_t)j * n + i] : 0.0;
    free(lt);
    return 0;
}

int imfcs_o_fit_gls(const double *acf, const double *covmats, const double *lagtime, int chanum,
                    const double *init, const int *free_mask, const double *cst, int max_iter,
                    double *out, double *chi2, double *cov, double *sigma, double *tres,
                    int *iters)
{
    int n = chanum - 1;
    double *L = (double *)malloc(sizeof(double) * n * n);
    double *y = (double *)malloc(sizeof(double) * n * (1 + IMFCS_O_NPARAM));
    double *jw = y + n;
    if (cm_cholesky(covmats, n, L)) {
        free(L); free(y);
        for (int i = 0; i < IMFCS_O_NPARAM; i++) out[i] = NAN;
        return 1;
    }
    for (int i = 0; i < n; i++) { /* transACF = L^-1 corav[1..] */
        double s = acf[i + 1];
        for (int m = 0; m < i; m++) s -= L[(size_t)i * n + m] * y[m];
        y[i] = s / L[(size_t)i * n + i];
    }
    fcs_ctx c;
    memset(&c, 0, sizeof(c));
    c.lagtime = lagtime + 1; c.n = n; c.init = init; c.free_mask = free_mask; c.cst = cst;
    c.linv = L;
    for (int i = 0; i < IMFCS_O_NPARAM; i++) if (free_mask[i]) c.idx[c.k++] = i;
    double p[IMFCS_O_NPARAM];
    for (int j = 0; j < c.k; j++) p[j] = init[c.idx[j]] / O_UNIT[c.idx[j]];
    lm_info info;
    int st = lm_solve(fcs_points, &c, n, c.k, y, NULL, p, max_iter, &info, jw);
    if (iters) *iters = info.iters;
    int fail = (st != 0) || param_cov(jw, n, c.k, c.idx, cov, sigma);
    if (fail) {
        for (int i = 0; i < IMFCS_O_NPARAM; i++) out[i] = NAN;
        free(L); free(y);
        return 1;
    }
    fcs_expand(&c, p, out);
    *chi2 = info.chi2 / (chanum - c.k - 1); /* java:10713-10715 */
    if (tres)
        for (int i = 1; i < chanum; i++) {
            double v; imfcs_o_fcs_model(out, cst, lagtime[i], &v, NULL);
            tres[i - 1] = acf[i] - v;
        }
    free(L); free(y);
    return 0;
}

/* determinant by cofactor expansion (java:14752-14789). */
static double o_det(const double *a, int n, int lda)
{
    if (n == 1) return a[0];
    if (n == 2) return a[0] * a[lda + 1] - a[lda] * a[1];
    double res = 0.0, m[64];
    for (int j1 = 0; j1 < n; j1++) {
        for (int i = 1; i < n; i++) {
            int j2 = 0;
            for (int j = 0; j < n; j++) {
                if (j == j1) continue;
                m[(i - 1) * (n - 1) + j2] = a[i * lda + j];
                j2++;
            }
        }
        res += pow(-1.0, 1.0 + j1 + 1.0) * a[j1] * o_det(m, n - 1, n - 1);
    }
    return res;
}

int imfcs_o_bayes(const double *acf, const double *var, const double *covmats,
                  const double *lagtime, int chanum, int fitstart, int fitend, int gls,
                  const double *init, const double *cst, int max_iter, double *prob2,
                  double *fit1, double *fit2)
{
    const double pi = O_PI;
    const int boxsize = 200;
    double modprob[2];
    int n1 = chanum - 1;
    double *tres = (double *)malloc(sizeof(double) * n1 * 2);
    double *sol = tres + n1;
    for (int model = 0; model < 2; model++) {
        double in[IMFCS_O_NPARAM] = {0};
        int fm[IMFCS_O_NPARAM] = {0};
        in[0] = init[0]; in[1] = init[1]; in[4] = init[4];
        fm[0] = fm[1] = fm[4] = 1;
        if (model == 1) { in[5] = 0.5; in[6] = 0.1 * init[1]; fm[5] = fm[6] = 1; }
        int numel = model == 0 ? 3 : 5;
        double cov[25], sigma[5], chi2, *out = model == 0 ? fit1 : fit2, logresid;
        int st;
        if (!gls) {
            st = imfcs_o_fit_ols(acf, var, lagtime, chanum, fitstart, fitend, in, fm, cst,
                                 max_iter, out, &chi2, cov, sigma, tres, NULL);
        } else {
            st = imfcs_o_fit_gls(acf, covmats, lagtime, chanum, in, fm, cst, max_iter, out,
                                 &chi2, cov, sigma, tres, NULL);
        }
        if (st) { /* failed fit: the Java catch block returns ones (java:10441-10466) */
            for (int i = 0; i < n1; i++) tres[i] = 1;
            for (int i = 0; i < numel * numel; i++) cov[i] = 1;
            for (int i = 0; i < numel; i++) sigma[i] = 1;
        }
        if (!gls) {
            double residsum = 0.0;
            for (int i = 1; i < n1; i++) residsum += tres[i] * tres[i]; /* starts at 1 (java:10170) */
            logresid = -0.5 * residsum;
        } else {
            /* solve covmats^T s = tres by LU with partial pivoting */
            double *a = (double *)malloc(sizeof(double) * n1 * n1);
            int *piv = (int *)malloc(sizeof(int) * n1);
            for (int i = 0; i < n1; i++)
                for (int j = 0; j < n1; j++) a[i * n1 + j] = covmats[j * n1 + i];
            for (int i = 0; i < n1; i++) { piv[i] = i; sol[i] = tres[i]; }
            for (int col = 0; col < n1; col++) {
                int pr = col;
                for (int r = col + 1; r < n1; r++) if (fabs(a[r * n1 + col]) > fabs(a[pr * n1 + col])) pr = r;
                if (pr != col) {
                    for (int j = 0; j < n1; j++) { double t = a[col * n1 + j]; a[col * n1 + j] = a[pr * n1 + j]; a[pr * n1 + j] = t; }
                    double t = sol[col]; sol[col] = sol[pr]; sol[pr] = t;
                }
                for (int r = col + 1; r < n1; r++) {
                    double fct = a[r * n1 + col] / a[col * n1 + col];
                    for (int j = col; j < n1; j++) a[r * n1 + j] -= fct * a[col * n1 + j];
                    sol[r] -= fct * sol[col];
                }
            }
            for (int i = n1 - 1; i >= 0; i--) {
                double s = sol[i];
                for (int j = i + 1; j < n1; j++) s -= a[i * n1 + j] * sol[j];
                sol[i] = s / a[i * n1 + i];
            }
            double d = 0.0;
            for (int i = 0; i < n1; i++) d += sol[i] * tres[i];
            logresid = -0.5 * d;
            free(a); free(piv);
        }
        double det = o_det(cov, numel, numel);
        double prodsigma = 1.0;
        for (int i = 0; i < numel; i++) prodsigma *= sigma[i];
        modprob[model] = exp(0.5 * numel * log(2 * pi) + 0.5 * log(det) + logresid -
                             log(prodsigma * pow(2 * boxsize, numel)));
    }
    double norm = modprob[0] + modprob[1];
    prob2[0] = modprob[0] / norm;
    prob2[1] = modprob[1] / norm;
    free(tres);
    return 0;
}

typedef struct { const double *x; int n; } line_ctx;
static void line_model(const double *p, double *f, double *jac, void *vctx)
{
    line_ctx *c = (line_ctx *)vctx;
    for (int i = 0; i < c->n; i++) {
        f[i] = p[0] + p[1] * c->x[i];
        jac[i * 2] = 1.0;
        jac[i * 2 + 1] = c->x[i];
    }
}

int imfcs_o_line_fit(const double *x, const double *y, const double *sd, int n, double *res2)
{
    double w[256];
    for (int i = 0; i < n; i++) w[i] = 1.0 / sd[i] / sd[i];
    res2[0] = y[0];                                   /* java:10814-10815 */
    res2[1] = (y[1] - y[0]) / (x[1] - x[0]);
    line_ctx c = {x, n};
    lm_info info;
    return lm_solve(line_model, &c, n, 2, y, w, res2, 100000, &info, NULL) == 2;
}

/* ------------------------------------------------------------------------ */
/* Whole path (correlateROI CPU loop java:8457-8556, correlate 9124-9200).   */
/* ------------------------------------------------------------------------ */
int imfcs_o_run(const imfcs_o_config *cfg, const uint16_t *stack, const int *bgr, double *acf,
                double *var, double *sd, int *blocked_ind, int *blocked_ok, double *fitres,
                double *chi2, int *fitted, double *bayes_prob, double *covmats)
{
    const int chanum = imfcs_o_chanum(cfg->p, cfg->q);
    const int num = cfg->num;
    const int npix = cfg->out_w * cfg->out_h;
    int *lag = (int *)malloc(sizeof(int) * chanum);
    double *samp = (double *)malloc(sizeof(double) * chanum);
    double *mtab = (double *)malloc(sizeof(double) * chanum);
    double *lagtime = (double *)malloc(sizeof(double) * chanum);
    imfcs_o_lag_tables(cfg->p, cfg->q, num, lag, samp, mtab);
    for (int i = 0; i < chanum; i++) lagtime[i] = lag[i] * cfg->frametime;
    int nopit = num < 1000 ? num : 1000;
    int err = 0;

#ifdef _OPENMP
    int nth = cfg->threads > 0 ? cfg->threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
#endif
    for (int pix = 0; pix < npix; pix++) {
        int ox = pix % cfg->out_w, oy = pix / cfg->out_w;
        int px1 = (cfg->map_x0 + ox) * cfg->pixbinx, py1 = (cfg->map_y0 + oy) * cfg->pixbiny;
        int px2 = px1 + cfg->cfx, py2 = py1 + cfg->cfy;
        int is_ccf = (px1 != px2 || py1 != py2);
        double *c0 = (double *)malloc(sizeof(double) * (num + 1) * 2);
        double *c1 = is_ccf ? c0 + num + 1 : c0;
        double tr[1000], tt[1000], res[16];
        double *covm = cfg->gls ? (double *)malloc(sizeof(double) * (chanum - 1) * (chanum - 1)) : NULL;
        for (int ch = 0; ch < (is_ccf ? 2 : 1); ch++) {
            int px = ch ? px2 : px1, py = ch ? py2 : py1;
            double *c = ch ? c1 : c0;
            imfcs_o_get_intensity(stack, cfg->width, cfg->height, cfg->first, num, px, py,
                                  cfg->binx, cfg->biny, cfg->background, bgr, c);
            if (cfg->bleach != IMFCS_O_BLEACH_NONE) {
                imfcs_o_intensity_trace(stack, cfg->width, cfg->height, cfg->first, num, px, py, px1, py1,
                                        cfg->binx, cfg->biny, cfg->background, bgr, nopit,
                                        cfg->frametime, tr, tt);
                int st = 0;
                if (cfg->bleach == IMFCS_O_BLEACH_POLY) {
                    st = imfcs_o_poly_fit(tr, tt, nopit, cfg->poly_order, res);
                    if (!st) imfcs_o_bleach_apply(c, num, cfg->frametime, cfg->bleach, cfg->poly_order, res);
                } else {
                    const int two = cfg->bleach == IMFCS_O_BLEACH_DOUBLE_EXP;
                    st = exp_fit_rate(tr, tt, nopit, two, res);
                    if (!st) bleach_apply_rate(c, num, cfg->frametime, two ? 2 : 1, res);
                }
            }
        }
        int bok = 0;
        int ind = imfcs_o_block_transform(c0, c1, num, cfg->p, cfg->q, lag, samp, mtab,
                                          cfg->frametime, &bok, NULL);
        double *a = acf + (size_t)pix * chanum, *v = var + (size_t)pix * chanum;
        double *s = sd + (size_t)pix * chanum;
        imfcs_o_calculate_cf(c0, c1, num, ind, cfg->p, cfg->q, lag, samp, mtab, cfg->gls, a, v, s, covm);
        blocked_ind[pix] = ind;
        blocked_ok[pix] = bok;
        if (covm && covmats)
            memcpy(covmats + (size_t)pix * (chanum - 1) * (chanum - 1), covm,
                   sizeof(double) * (chanum - 1) * (chanum - 1));
        if (cfg->do_fit) {
            double *fr = fitres + (size_t)pix * IMFCS_O_NPARAM, x2 = NAN;
            int st;
            if (cfg->gls)
                st = imfcs_o_fit_gls(a, covm, lagtime, chanum, cfg->init, cfg->free_mask, cfg->cst,
                                     cfg->max_iter, fr, &x2, NULL, NULL, NULL, NULL);
            else
                st = imfcs_o_fit_ols(a, v, lagtime, chanum, cfg->fitstart, cfg->fitend, cfg->init,
                                     cfg->free_mask, cfg->cst, cfg->max_iter, fr, &x2, NULL, NULL,
                                     NULL, NULL);
            chi2[pix] = x2;
            fitted[pix] = (st == 0);
            if (cfg->bayes && bayes_prob) {
                double f1[IMFCS_O_NPARAM], f2[IMFCS_O_NPARAM];
                imfcs_o_bayes(a, v, covm, lagtime, chanum, cfg->fitstart, cfg->fitend, cfg->gls,
                              cfg->init, cfg->cst, cfg->max_iter, bayes_prob + 2 * (size_t)pix, f1, f2);
            }
        }
        free(c0);
        free(covm);
    }
    free(lag); free(samp); free(mtab); free(lagtime);
    return err;
}
