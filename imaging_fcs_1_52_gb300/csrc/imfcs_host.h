// imfcs_host.h -- host-side declarations shared by the C-ABI translation units.
#pragma once

#include <string>

#include "imfcs_internal.cuh"
#include "imfcs_gb300.h"

namespace imfcs {

// launchers (defined in the kernel translation units)
cudaError_t launch_corr(const Job &j, const LagInfo *li, const void *stack, const float *bparams,
                        const float *basis, const float *s0, const float4 *mon, const int *blk_ind, double *acf,
                        double *var, double *sd, double *nb_mean, double *nb_cov, float *bprod,
                        int pnum_stride, float *stats, float *streams, int gls, int *err,
                        cudaStream_t stream);
size_t corr_smem_bytes(int q, bool ccf);
size_t corr_stats_floats(const Job &j);    // per-lag block statistics scratch (floats)
size_t corr_stream_floats(const Job &j);   // binned sample streams of the correlator chain (floats)
size_t level0_stream_floats(const Job &j); // the corrected level-0 stream s0 (floats)
int corr_kernel_count(const Job &j);        // kernels one correlator launch issues

struct FitArgs;
cudaError_t launch_lm(const FitArgs &a, int num_sms, cudaStream_t stream);
struct EpilogueArgs;
cudaError_t launch_fit_epilogue(const EpilogueArgs &e, cudaStream_t stream);
cudaError_t launch_ols_prepare(int npix, int chanum, int fitstart, int npts, const double *acf,
                               const double *var, float *y, float *w, cudaStream_t stream);
cudaError_t launch_bayes_combine(int npix, const double *lp1, const double *lp2, float *prob,
                                 cudaStream_t stream);
struct GlsArgs;
cudaError_t launch_gls(const GlsArgs &g, cudaStream_t stream);

// prep launchers (imfcs_prep_launch.cu)
cudaError_t launch_trace(const Job &j, const void *stack, float *trace, cudaStream_t s);
cudaError_t launch_bleach(const Job &j, const float *trace, const double *proj, float uscale,
                          float uoff, float *bparams, cudaStream_t s);
cudaError_t launch_center_given(const Job &j, const float *trace, float *bparams, cudaStream_t s);
cudaError_t launch_stream(const Job &j, const void *stack, const float *bparams, const float *basis,
                          const int *snap_pos, int nseg, float *s0, float2 *segtot, float2 *snap_part, int *segbad,
                          int *snap_bad, int *err, cudaStream_t s);
cudaError_t launch_monitor_finalize(const Job &j, const LagInfo *li_dev, const float *bparams, int nseg,
                                    const float2 *segtot, const float2 *snap_part, const int *segbad,
                                    const int *snap_bad, float4 *mon, float4 *blkmon, cudaStream_t s);
// N&B mode: lag-1 mean and covariance only (sum: npix doubles of scratch)
cudaError_t launch_nb_lag1(const Job &j, const float *s0, const float4 *mon, double *sum, double *nb_mean,
                           double *nb_cov, cudaStream_t s);
cudaError_t launch_block(const Job &j, const float *s0, const float4 *blkmon, int nbseg, float *s1, float *s2,
                         float *segsum, int *ind, int *ok, cudaStream_t s);
cudaError_t launch_binning(const float *in, float *out, int win, int hin, int wt, int ht,
                           int frames, int bx, int by, cudaStream_t s);
cudaError_t launch_bleach_average(const float *in, float *out, int w, int h, int nopit, int ave,
                                  cudaStream_t s);

// surrogate seeds (imfcs_mlp.cu): features, prediction and per-pixel LM
// initial values init[pix][11] from the shared base_init (internal units)
// (free parameters idx[0..k) only)
int surrogate_seed(imfcs_surrogate *h, int npix, int chanum, int k, const int *idx, const double *acf,
                   const double *var, float *x, float *pred, const float *base_init, float *init, cudaStream_t s);
int surrogate_reserve(imfcs_surrogate *h, int n);   // work buffers for n pixels (allocates)
// refit decision after a seeded LM: todo[pix] = 1 where the pixel's fit data
// y/w [pix][npts] are finite and the seeded fit did not converge, ended with
// N <= 0, D <= 0 or a non-finite free parameter, or (plain_chi2 given) its
// chi^2 exceeds the converged plain chi^2 by > 1 %; counts[0] += refits,
// counts[1] += the chi^2 cases
cudaError_t launch_seed_select(int npix, int k, const int *idx, const float *par, const int *state,
                               const float *chi2, const int *plain_state, const float *plain_chi2, const float *y,
                               const float *w, int npts, int *todo, int *counts, cudaStream_t s);

// error state
void set_error(const std::string &msg);
std::string cuda_msg(cudaError_t e, const char *what);

// Lag-table and structure set-up shared by the plan and the reference calcACF.
bool build_lag_info(int p, int q, int num, LagInfo &li, int &chanum, int &blocknum,
                    std::string &err);

// Legendre projection for the polynomial bleach fit: proj[(order+1)][nopit]
// (FP64, host), and the u-mapping of time.
void legendre_projection(int order, int nopit, int ave, double frametime, double *proj,
                         double &uscale, double &uoff);
void legendre_basis_table(int order, int num, double frametime, double uscale, double uoff,
                          float *table);

// the checks imfcs_plan_create applies to a configuration
bool config_valid(const imfcs_config *c, std::string &err);

// external_scratch: the plan's per-execution scratch is not allocated; a
// batch binds an arena of plan_scratch_need bytes before each execution
int plan_create_ex(const imfcs_config *cfg, int input_float, int in_w, int in_h, bool given_bleach,
                   imfcs_plan **plan_out, bool external_scratch = false);
int plan_execute_any(imfcs_plan *pl, const void *dev_stack, const imfcs_outputs *dev_out, void *stream);
bool corr2_supported(const Job &j);          // the level chain runs (P = 16, Q >= 5)

// batch support (imfcs_batch.cu): per-execution scratch bytes, binding an
// arena, the plan's device error flag, the correlator alone
size_t plan_scratch_need(const imfcs_plan *pl);
void plan_bind_scratch(imfcs_plan *pl, void *base);
const int *plan_dev_err(const imfcs_plan *pl);
const Job &plan_job(imfcs_plan *pl);
int plan_corr_only(imfcs_plan *pl, const void *dev_stack, const imfcs_outputs *dev_out, cudaStream_t s);

}  // namespace imfcs
