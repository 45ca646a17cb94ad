/*
 * imfcs_oracle.h -- FP64 CPU restatement of the Imaging_FCS 1.52 Java CPU path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine
 * (tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * arm).  It is never linked into, loaded by, or called from the product
 * library (libimfcs_gb300.so).
 *
 * Parity status: the reference ships no tests, fixtures or golden vectors,
 * and its Java path cannot run here (no JVM, no ImageJ/commons-math jars).
 * This restatement is pinned only by the documented lag-table example of the
 * reference manual, by analytic cases (constant trace, white noise, closed
 * form model values) and by MINPACK (scipy) for the least-squares minimum:
 * parity of the correlator and fit numerics against the Java code itself is
 * UNPINNED.
 *
 * Every function cites the Java lines it restates (Imaging_FCS_1_52.java).
 */
#ifndef IMFCS_ORACLE_H
#define IMFCS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IMFCS_O_NPARAM 11   /* N, D, vx, vy, G, F2, D2, F3, D3, Ftrip, Ttrip */
#define IMFCS_O_NCONST 9    /* ax, ay, s, sz, rx, ry, fitobsvol, q2, q3     */

enum { IMFCS_O_BLEACH_NONE = 0, IMFCS_O_BLEACH_SINGLE_EXP = 1,
       IMFCS_O_BLEACH_DOUBLE_EXP = 2, IMFCS_O_BLEACH_POLY = 3 };

/* Lag tables: setParameters, Imaging_FCS_1_52.java:7340-7346, 7391-7424. */
int  imfcs_o_chanum(int p, int q);
void imfcs_o_lag_tables(int p, int q, int num, int *lag, double *samp, double *mtab);

/* getIntensity (Imaging_FCS_1_52.java:9651-9678): 1-based trace out[0..num],
 * out[0] = 0.  stack is [frames][height][width] uint16; bgr (optional,
 * [height][width] ints) replaces the scalar background per raw pixel. */
void imfcs_o_get_intensity(const uint16_t *stack, int width, int height, int first,
                           int num, int px, int py, int binx, int biny, int bckg,
                           const int *bgr, double *out);

/* calcIntensityTrace (Imaging_FCS_1_52.java:9822-9855): nopit averages with
 * Java int division; trace_time = frametime*(x+0.5)*ave.  The background
 * image (bgr) is read at the window (bgx, bgy): the direct window for both
 * traces of a cross-correlation, as java:9842-9845 does. */
void imfcs_o_intensity_trace(const uint16_t *stack, int width, int height, int first,
                             int num, int px, int py, int bgx, int bgy, int binx, int biny,
                             int bckg, const int *bgr, int nopit, double frametime,
                             double *trace, double *trace_time);

/* Bleach fits on the averaged trace.  PolynomFit (java:10953-11004),
 * SingleExpFit (java:10845-10895), DoubleExpFit (java:10898-10950).
 * Return 0 on success. */
int imfcs_o_poly_fit(const double *y, const double *t, int n, int order, double *coef);
int imfcs_o_exp_fit(const double *y, const double *t, int n, double *res3);
int imfcs_o_dexp_fit(const double *y, const double *t, int n, double *res5);

/* Exponential fits in the rate form f0 - sum s_c (1 - e^{-k_c t}) / k_c,
 * k_c >= 0, with the standard errors of (f0, s1, k1 [, s2, k2]). */
int imfcs_o_exp_fit_rate(const double *y, const double *t, int n, int two, double *rate, double *sigma);

/* Correction of the 1-based trace (java:9682-9769). */
void imfcs_o_bleach_apply(double *intdat, int num, double frametime, int mode,
                          int order, const double *res);

/* blockTransform (java:9217-9422).  c0/c1 are the 1-based traces; like the
 * Java code, elements [0..num-1] are read.  Returns ind, writes blockIndS.
 * varblock (optional) receives [3][blocknum]. */
int imfcs_o_block_transform(const double *c0, const double *c1, int num, int p, int q,
                            const int *lag, const double *samp, const double *mtab,
                            double frametime, int *block_ind_s, double *varblock);

/* calculateCF (java:9425-9648).  Elements [1..num] are read.  Outputs have
 * chanum entries; covmats ((chanum-1)^2) only when gls != 0.  When gls != 0,
 * corav receives mcov, as in the Java code. */
void imfcs_o_calculate_cf(const double *c0, const double *c1, int num, int ind, int p,
                          int q, const int *lag, const double *samp, const double *mtab,
                          int gls, double *corav, double *blockvar, double *blocksd,
                          double *covmats);

/* FCS_3p value and gradient (java:13131-13408) for one lag time. */
void imfcs_o_fcs_model(const double *par, const double *cst, double tau, double *value,
                       double *grad);

/* obsvolFCS_ST2D1p(2) (java:13670-13702). */
double imfcs_o_obsvol(double ax, double ay, double s);

/* standardFit (java:10288-10471): weighted LM over lags fitstart..fitend.
 * Outputs: out[11] (held parameters keep their init values), chi2 (reduced,
 * as java:10403-10406), cov (KxK, (J^T J)^-1 of the weighted problem),
 * sigma (K), tres (chanum-1 unweighted residuals, zero outside range).
 * Returns 0 on success, nonzero when the fit failed. */
int imfcs_o_fit_ols(const double *acf, const double *var, const double *lagtime,
                    int chanum, int fitstart, int fitend, const double *init,
                    const int *free_mask, const double *cst, int max_iter, double *out,
                    double *chi2, double *cov, double *sigma, double *tres, int *iters);

/* dataTransform + GLSFit (java:13705-13729, 10622-10789, 13569-13666). */
int imfcs_o_fit_gls(const double *acf, const double *covmats, const double *lagtime,
                    int chanum, const double *init, const int *free_mask,
                    const double *cst, int max_iter, double *out, double *chi2,
                    double *cov, double *sigma, double *tres, int *iters);

/* bayesFit (java:10094-10285): model probabilities of 1 and 2 components. */
int imfcs_o_bayes(const double *acf, const double *var, const double *covmats,
                  const double *lagtime, int chanum, int fitstart, int fitend, int gls,
                  const double *init, const double *cst, int max_iter, double *prob2,
                  double *fit1, double *fit2);

/* LineFit (java:10792-10842) with weights 1/sd^2. */
int imfcs_o_line_fit(const double *x, const double *y, const double *sd, int n,
                     double *res2);

/* Whole path over an output grid (correlateROI CPU loop, java:8457-8556).
 * Layout of outputs: [pixel][chanum] with pixel = oy*out_w + ox. */
typedef struct {
    int width, height, frames;   /* raw stack [frames][height][width] */
    int first, num;              /* 0-based first frame and number of frames */
    int out_w, out_h;            /* output grid */
    int map_x0, map_y0;          /* map offset of output (0,0) */
    int binx, biny, pixbinx, pixbiny;
    int cfx, cfy;
    int background;
    int p, q;
    double frametime;
    int bleach, poly_order;
    int gls, bayes, do_fit;
    int fitstart, fitend;
    int max_iter;
    double init[IMFCS_O_NPARAM];
    int free_mask[IMFCS_O_NPARAM];
    double cst[IMFCS_O_NCONST];
    int threads;                 /* OpenMP threads, <=0: all */
} imfcs_o_config;

int imfcs_o_run(const imfcs_o_config *cfg, const uint16_t *stack, const int *bgr,
                double *acf, double *var, double *sd, int *blocked_ind, int *blocked_ok,
                double *fitres, double *chi2, int *fitted, double *bayes_prob,
                double *covmats /* [pixel][(chanum-1)^2] when gls, nullable */);

#ifdef __cplusplus
}
#endif
#endif
