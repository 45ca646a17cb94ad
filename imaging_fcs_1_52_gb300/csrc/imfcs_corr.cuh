// imfcs_corr.cuh -- outputs and per-lag block statistics shared by the
// correlator kernels.
#pragma once

#include "imfcs_internal.cuh"

namespace imfcs {

constexpr int kStatN = 5;   // per-lag block statistics: Ahi, Alo (float-float product total), S1, S2, r

struct CorrOut {
    double *acf, *var, *sd;
    double *nb_mean, *nb_cov;
    float *bprod;        // GLS: [pix][chanum-1][pnum_max]
    int pnum_stride;
    float *stats;        // scratch [chanum][kStatN][npix]
    int gls;
    int *err;            // set to 1 when a bounded wait gave up
};

__device__ __forceinline__ float &stat_ref(float *stats, int npix, int lag, int s, int pix)
{
    return stats[((size_t)lag * kStatN + s) * npix + pix];
}

}  // namespace imfcs
