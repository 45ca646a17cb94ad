/*
 * fake_imfcs.c -- a recording stand-in for the library's reference-facing
 * C ABI, linked under jni/imfcs_jni.c in the CPU tests: every entry point the
 * shim calls records its arguments, writes a marker into its outputs and
 * returns the code the test set, so the tests see exactly what the shim
 * passes and what it copies back -- without a GPU.
 */
#include <string.h>

#include "imfcs_gb300.h"

static int g_rc;
static imfcs_acf_parameters g_params;
static const void *g_ptrs[16];
static long g_ints[16];
static float g_tol;
static char g_last[64] = "";

void fake_set_rc(int rc) { g_rc = rc; }
void fake_params(imfcs_acf_parameters *out) { *out = g_params; }
const void *fake_ptr(int i) { return (i >= 0 && i < 16) ? g_ptrs[i] : NULL; }
long fake_int(int i) { return (i >= 0 && i < 16) ? g_ints[i] : 0; }
float fake_tol(void) { return g_tol; }
const char *fake_last_call(void) { return g_last; }

static int finish(const char *name)
{
    strncpy(g_last, name, sizeof(g_last) - 1);
    return g_rc;
}

const char *imfcs_get_last_error(void) { return g_rc ? "fake failure" : ""; }
int imfcs_is_cuda_available(void) { return g_rc == 0; }
int imfcs_get_cuda_version(int *rt, int *dr)
{
    *rt = 13000;
    *dr = 13000;
    return finish("version");
}
int imfcs_reset_gpu(void) { return finish("reset"); }
int imfcs_is_binning_memory_sufficient(const imfcs_acf_parameters *p)
{
    g_params = *p;
    finish("binmem");
    return g_rc == 0;
}
int imfcs_is_acf_memory_sufficient(const imfcs_acf_parameters *p)
{
    g_params = *p;
    finish("acfmem");
    return g_rc == 0;
}
int imfcs_calc_binning(const float *in, float *out, const imfcs_acf_parameters *p)
{
    g_params = *p;
    g_ptrs[0] = in;
    g_ptrs[1] = out;
    if (out) out[0] = in ? in[0] + 1.f : -1.f;
    return finish("binning");
}
int imfcs_calc_data_bleach_correction(const float *px, float *out, const imfcs_acf_parameters *p)
{
    g_params = *p;
    g_ptrs[0] = px;
    g_ptrs[1] = out;
    if (out) out[0] = 7.f;
    return finish("bleachavg");
}
int imfcs_calc_acf(const float *pixels, double *acf, double *var, double *nbm, double *nbc, double *blk,
                   const double *bcp, double *samp, int *lag, const imfcs_acf_parameters *p)
{
    g_params = *p;
    const void *ptrs[9] = {pixels, acf, var, nbm, nbc, blk, bcp, samp, lag};
    memcpy(g_ptrs, ptrs, sizeof(ptrs));
    g_ints[0] = pixels ? (long)pixels[0] : -1;
    g_ints[1] = bcp ? (long)bcp[0] : -1;
    if (acf) acf[0] = 1.5;
    if (var) var[0] = 2.5;
    if (nbm) nbm[0] = 3.5;
    if (nbc) nbc[0] = 4.5;
    if (blk) blk[0] = 5.5;
    if (samp) samp[0] = 6.5;
    if (lag) lag[0] = 7;
    return finish("acf");
}
int imfcs_fit(int n_fits, int n_points, const float *data, const float *weights, int model_id,
              const float *init, float tol, int max_iter, int ncoef, const int *to_fit, int estimator,
              size_t ui_size, const void *ui, float *out_par, int *out_states, float *out_chi2, int *out_iter)
{
    const void *ptrs[10] = {data, weights, init, to_fit, ui, out_par, out_states, out_chi2, out_iter, NULL};
    memcpy(g_ptrs, ptrs, sizeof(ptrs));
    long ints[7] = {n_fits, n_points, model_id, max_iter, ncoef, estimator, (long)ui_size};
    memcpy(g_ints, ints, sizeof(ints));
    g_tol = tol;
    return finish("fit");
}
