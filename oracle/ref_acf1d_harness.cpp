// ref_acf1d_harness.cpp -- host-side harness around the reference's own
// ACF_1D model function (calculate_acf1d, agpufitjni.cu:427-543), which the
// oracle Makefile's `ref` target extracts from the reference source into
// oracle/_ref/ (never committed).  TEST INFRASTRUCTURE ONLY: it pins the
// oracle's FCS_3p restatement against the reference's compiled model code.
#include <cmath>
#include <cstddef>

#define __device__
typedef float REAL;

#include "acf1d_extract.inc"

// params20: the 20 Gpufit ACF_1D parameters (N, D, vx, vy, G, F2, D2, F3, D3,
// Ftrip, Ttrip, ax, ay, s, sz, rx, ry, fitobsvol, q2, q3; SI units); x: lag
// times (s).  value[npts], deriv[20][npts] (rows the reference does not set
// are left as given).
extern "C" void ref_acf1d(const float *params20, int npts, const float *x, float *value, float *deriv)
{
    for (int i = 0; i < npts; i++)
        calculate_acf1d(params20, 1, npts, value, deriv, i, 0, 0, (char *)x, sizeof(float) * npts, 0);
}
