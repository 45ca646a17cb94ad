// imfcs_args.h -- argument blocks of the fit and GLS kernels (shared with the host).
#pragma once

#include "imfcs_internal.cuh"

namespace imfcs {

struct FitArgs {
    int nfits, npts;
    int model;               // IMFCS_MODEL_ACF_1D or IMFCS_MODEL_LINEAR_1D
    int np;                  // parameters in the full vector (11 for ACF, coefs for LINEAR)
    int k, idx[IMFCS_NPARAM];
    int max_iter;
    float tol;               // > 0: Gpufit convergence test; 0: step test
    // data
    const float *y;          // [fit][npts]
    const float *w;          // [fit][npts] or nullptr (unit weights)
    const float *x;          // [npts] abscissae (lag times s / polynomial x)
    const float *init;       // [fit][init_stride] internal units, or shared when init_stride == 0
    int init_stride;
    const float *cst;        // [fit][9] per-fit constants (SI -> internal on load) or nullptr
    ModelConst mc;           // shared constants when cst == nullptr
    // GLS
    const float *linv;       // [fit][npts*(npts+1)/2] packed lower L^-1, or nullptr
    // outputs
    float *out_par;          // [fit][out_stride] (internal units)
    int out_stride;
    float *out_chi2;         // raw weighted chi^2
    int *out_state;
    int *out_iter;
    float *out_hess;         // [fit][k*k] J^T W J at the optimum (internal units) or nullptr
    const int *todo;         // [fit]: 0 = leave this fit's outputs untouched; nullptr = fit all
    int *counter;            // zeroed work counter: warps take fits dynamically; nullptr = static stride
    int tirf_zero_held;      // the held parameters (vx, vy, F2, F3, Ftrip) are zero for every fit
};

struct EpilogueArgs {
    int npix, chanum, npts, k, idx[IMFCS_NPARAM];
    int fitstart, fitend;
    int gls;
    double chi2_div;             // (fitend - fitstart) - k - 1  or  chanum - k - 1
    const float *par_int;        // [pix][11] internal
    const float *chi2_raw;
    const int *state;
    const float *hess;           // [pix][k*k] internal
    float *fitres;               // [pix][11] SI
    float *chi2;
    int *fitted;
    double *logp;                // [pix] Bayes log-probability term (nullable)
    const int *pre_ok;           // [pix] GLS factorisation succeeded (nullable)
    const double *acf;           // for residuals
    const float *linv;           // GLS
    ModelConst mc;
    const float *lagtime;        // [chanum]
};

struct GlsArgs {
    int npix, chanum, pnum_stride;
    const float *bprod;      // [pix][chanum-1][pnum_stride]
    const float4 *mon;       // [pix][chanum]
    const int *blk_ind;
    const int *pnum_by_ind;  // device copy
    float *linv;             // [pix][n1*(n1+1)/2]
    float *ytrans;           // [pix][n1]  L^-1 mcov[1..]
    int *ok;                 // [pix]
    double *covmats_out;     // [pix][n1*n1] or nullptr
};

}  // namespace imfcs
