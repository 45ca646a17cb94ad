// imfcs_ff.cuh -- float-float ("double-single") arithmetic on the FP32
// pipes: a value is hi + lo with |lo| <= ulp(hi)/2, about 48 significant bits.
// Exact two-sum (Knuth) and two-product (FMA), with explicitly rounded
// operations so that the compiler cannot contract or reassociate them.
// GB300 issues FP64 at 1/64 of the FP32 rate; a float-float operation costs
// a handful of FP32 ones.
#pragma once

namespace imfcs {

struct f2 {
    float hi, lo;
};
__device__ __forceinline__ f2 f2_quick(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ f2 f2_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ f2 f2_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 s = f2_two_sum(a.hi, b.hi);
    return f2_quick(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ f2 f2_neg(f2 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 p = f2_two_prod(a.hi, b.hi);
    return f2_quick(p.hi, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo)));
}
__device__ __forceinline__ f2 f2_from_d(double x)
{
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

__device__ __forceinline__ f2 f2_from_f(float x) { return {x, 0.f}; }
// a * b with b a float
__device__ __forceinline__ f2 f2_mul_f(f2 a, float b)
{
    f2 p = f2_two_prod(a.hi, b);
    return f2_quick(p.hi, fmaf(a.lo, b, p.lo));
}
__device__ __forceinline__ float f2_val(f2 a) { return a.hi + a.lo; }

}  // namespace imfcs
