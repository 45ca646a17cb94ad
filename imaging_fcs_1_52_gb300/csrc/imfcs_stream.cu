// imfcs_stream.cu -- the one streaming pass over the raw uint16 stack after
// the bleach fit: every (trace, frame) is binned, background-subtracted,
// bleach-corrected (java:9682-9769) and centred once, written as the FP32
// level-0 sample stream s0[t][pixel] that the blocking transform and the
// correlator chain read, and summed into the monitor partials (float-float
// segment totals, the partial sums at every snapshot position the lags'
// windows need, and the count of non-finite frames) in the same pass.
//
// Staging: one CTA covers 32*NW consecutive output pixels of one output row
// and kStSegs monitor segments of kSeg = 256 frames.  Its raw frames arrive
// as TMA boxes [64 frames][bh rows][bw columns] (cp.async.bulk.tensor) in a
// ring of kStRing buffers, each completing on its own mbarrier; the threads
// (one per pixel) walk the staged frames in order.  Geometries TMA
// cannot take (float input, a row stride or base not 16-byte aligned, a box
// wider than 256) read the raw frames with plain loads instead.
//
// The exponential bleach curve is advanced by a recurrence e <- e q within
// each 64-frame stage (reseeded with exp() per stage: at most 64 FP32
// factors, ~4e-6 relative, a smooth factor that the normalised correlation
// does not see).  Non-finite corrected frames (a bleach curve through zero)
// are written as 0 and counted, so that the monitor finaliser makes exactly
// the lags whose windows hold one non-finite (calculateCF's NaN propagation,
// java:9484-9511).
//
// Waits are bounded (imfcs_tma.cuh): on a timeout the CTA records the error
// flag, waits (bounded) for its own copies and leaves.
#include <string.h>

#include "imfcs_host.h"
#include "imfcs_internal.cuh"
#include "imfcs_tma.cuh"

namespace imfcs {

constexpr int kStF = 64;                       // frames per TMA box
constexpr int kStRing = 3;                     // boxes in flight / being processed per CTA
constexpr int kStSegs = 4;                     // monitor segments per CTA
static_assert(kSeg % kStF == 0, "monitor segments must hold whole boxes");

struct StreamArgs {
    Job j;
    const void *stack;
    const float *bparams, *basis;
    const int *snap_pos;
    int nseg;
    float *s0a, *s0b;
    float2 *segtot, *snap_part;
    int *segbad, *snap_bad;
    int *err;
    int nw, tiles_x, bw, bh;   // TMA geometry (tma kernels)
};

// Correction state of one trace (bleach parameters, centre, recurrence).
template <int MODE>
struct StreamCorr {
    float f0, inv_f0, centre, c, k0, a0, k1, a1, q0, q1, e0, e1;
    int flags;
    bool on;
    float coef[kMaxPoly + 1];
    __device__ __forceinline__ void load(const float *bp, float frametime)
    {
        centre = __ldg(&bp[12]);
        on = MODE != IMFCS_BLEACH_NONE && __ldg(&bp[11]) != 0.f;
        f0 = __ldg(&bp[9]);
        inv_f0 = __ldg(&bp[10]);
        if (MODE == IMFCS_BLEACH_SINGLE_EXP || MODE == IMFCS_BLEACH_DOUBLE_EXP) {
            c = __ldg(&bp[13]);
            flags = (int)__ldg(&bp[14]);
            k0 = __ldg(&bp[5]);
            a0 = __ldg(&bp[7]);
            k1 = __ldg(&bp[6]);
            a1 = __ldg(&bp[8]);
            q0 = __expf(-k0 * frametime);
            q1 = __expf(-k1 * frametime);
        }
        if (MODE == IMFCS_BLEACH_POLYNOMIAL)
#pragma unroll
            for (int i = 0; i <= kMaxPoly; i++) coef[i] = __ldg(&bp[i]);
    }
    __device__ __forceinline__ void seed(int t, float frametime)
    {
        if (MODE == IMFCS_BLEACH_SINGLE_EXP || MODE == IMFCS_BLEACH_DOUBLE_EXP) {
            const float ft = frametime * ((float)t + 1.5f);   // java:9747, 1-based frame number
            e0 = __expf(-k0 * ft);
            if (MODE == IMFCS_BLEACH_DOUBLE_EXP) e1 = __expf(-k1 * ft);
        }
    }
    // corrected, centred value of raw window value v at frame t (the frame
    // after the previous call's, or the seeded one)
    __device__ __forceinline__ float apply(float v, int t, float frametime, int order, const float *basis)
    {
        if (MODE != IMFCS_BLEACH_NONE && on) {
            float f;
            if (MODE == IMFCS_BLEACH_POLYNOMIAL) {
                const float *b = basis + (size_t)t * (order + 1);
                f = 0.f;
                for (int i = 0; i <= order; i++) f = fmaf(coef[i], __ldg(&b[i]), f);
            } else {
                const float ft = frametime * ((float)t + 1.5f);
                f = c + ((flags & 1) ? -a0 * slow_exp_term(k0, ft) : a0 * e0);
                if (MODE == IMFCS_BLEACH_DOUBLE_EXP)
                    f += ((flags >> 1) & 1) ? -a1 * slow_exp_term(k1, ft) : a1 * e1;
            }
            v = bleach_correct(v, f, f0, inv_f0);
        }
        if (MODE == IMFCS_BLEACH_SINGLE_EXP || MODE == IMFCS_BLEACH_DOUBLE_EXP) {
            e0 *= q0;
            if (MODE == IMFCS_BLEACH_DOUBLE_EXP) e1 *= q1;
        }
        return v - centre;
    }
};

// Monitor partials of one trace over its segment.
struct MonAcc {
    ff acc;
    int bad, sj, next;
    __device__ __forceinline__ void init(const StreamArgs &a, int t0)
    {
        acc = {0.f, 0.f};
        bad = 0;
        int lo = 0, hi = a.j.nsnap;     // first snapshot with position > t0
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(&a.snap_pos[mid]) <= t0) lo = mid + 1; else hi = mid;
        }
        sj = lo;
        next = sj < a.j.nsnap ? __ldg(&a.snap_pos[sj]) : 0x7fffffff;
    }
    // value x of frame t; returns the value to store (0 when non-finite)
    __device__ __forceinline__ float add(const StreamArgs &a, int trace, int t, float x)
    {
        const bool fin = isfinite(x);
        if (fin) ff_add(acc, x); else bad++;
        while (t + 1 == next) {
            a.snap_part[(size_t)trace * a.j.nsnap + sj] = make_float2(acc.hi, acc.lo);
            a.snap_bad[(size_t)trace * a.j.nsnap + sj] = bad;
            sj++;
            next = sj < a.j.nsnap ? __ldg(&a.snap_pos[sj]) : 0x7fffffff;
        }
        return fin ? x : 0.f;
    }
    __device__ __forceinline__ void store(const StreamArgs &a, int trace, int seg)
    {
        a.segtot[(size_t)trace * a.nseg + seg] = make_float2(acc.hi, acc.lo);
        a.segbad[(size_t)trace * a.nseg + seg] = bad;
    }
};

// TMA-staged stream pass: grid (tiles_x * out_h, ceil(nseg / kStSegs)),
// 32 * nw threads.  A CTA walks kStSegs monitor segments (kStSegs * kSeg
// frames) through a ring of kStRing boxes: while one box is processed the
// next ones are in flight; a CTA barrier frees a box before thread 0 reloads
// it.  The outcome of every bounded wait is made uniform across the CTA
// (__syncthreads_or), so no thread is left waiting at a barrier.
template <int MODE, bool CCF, bool BIN1>
__global__ void __launch_bounds__(128) stream_tma_kernel(StreamArgs a, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) unsigned char ssm[];
    __shared__ uint64_t full[kStRing];
    const Job &j = a.j;
    const int nt = 32 * a.nw, tid = threadIdx.x;
    const int row = blockIdx.x / a.tiles_x, ox0 = (blockIdx.x % a.tiles_x) * nt;
    const int seg0 = blockIdx.y * kStSegs, seg1 = min(seg0 + kStSegs, a.nseg);
    const int t0 = seg0 * kSeg, t1 = min(seg1 * kSeg, j.num);
    const int box = kStF * a.bh * a.bw;
    uint16_t *tiles = (uint16_t *)ssm;
    const int rx0 = (j.map_x0 + ox0) * j.pixbinx + min(0, j.cfx);
    const int ry0 = (j.map_y0 + row) * j.pixbiny + min(0, j.cfy);
    const int tx0 = rx0 & ~7, xoff = rx0 - tx0;       // x rounded down to 16 bytes
    const int nbox = (t1 - t0 + kStF - 1) / kStF;
    if (tid == 0) {
        for (int b = 0; b < kStRing; b++) mbar_init(&full[b], 1);
        for (int b = 0; b < nbox && b < kStRing; b++)
            tma_load_box(&tmap, tiles + (size_t)b * box, &full[b], tx0, ry0, j.first + t0 + b * kStF,
                         (uint32_t)box * 2);
    }
    __syncthreads();
    const int ox = ox0 + tid;
    const bool valid = ox < j.out_w;
    const int pix = row * j.out_w + (valid ? ox : 0);
    const int xa = xoff + tid * j.pixbinx + (j.cfx < 0 ? -j.cfx : 0), ya = (j.cfy < 0 ? -j.cfy : 0);
    const int xb = xa + j.cfx, yb = ya + j.cfy;
    const int bga = trace_bg(j, pix), bgb = CCF ? trace_bg(j, j.npix + pix) : 0;
    StreamCorr<MODE> ca, cb;
    ca.load(a.bparams + (size_t)pix * kBleachStride, j.frametime);
    if (CCF) cb.load(a.bparams + (size_t)(j.npix + pix) * kBleachStride, j.frametime);
    MonAcc ma, mb;
    int issued = nbox < kStRing ? nbox : kStRing;
    for (int b = 0; b < nbox; b++) {
        const int slot = b % kStRing;
        const bool waited = mbar_wait(&full[slot], (uint32_t)((b / kStRing) & 1));
        if (__syncthreads_or(!waited)) {
            if (tid == 0) {
                atomicExch(a.err, 1);
                // the copies still in flight land before the CTA leaves
                for (int q = b; q < issued; q++) mbar_wait(&full[q % kStRing], (uint32_t)((q / kStRing) & 1));
            }
            return;
        }
        const int tb = t0 + b * kStF;
        const int seg = tb / kSeg;
        if (valid) {
            if (tb % kSeg == 0) {
                ma.init(a, tb);
                if (CCF) mb.init(a, tb);
            }
            ca.seed(tb, j.frametime);
            if (CCF) cb.seed(tb, j.frametime);
            const uint16_t *fa = tiles + (size_t)slot * box + ya * a.bw + xa;
            const uint16_t *fb = tiles + (size_t)slot * box + yb * a.bw + xb;
            const int n = min(kStF, t1 - tb);
            const int fstride = a.bh * a.bw;
            float *da = a.s0a + (size_t)tb * j.npix + pix, *db = a.s0b + (size_t)tb * j.npix + pix;
            if (BIN1 && n == kStF) {
                // a full box of unbinned windows: one shared-memory load per
                // frame and trace, the frame loop unrolled
#pragma unroll 8
                for (int f = 0; f < kStF; f++) {
                    const int t = tb + f;
                    const float va = ma.add(a, pix, t, ca.apply((float)((int)fa[f * fstride] - bga), t, j.frametime,
                                                                j.poly_order, a.basis));
                    da[(size_t)f * j.npix] = va;
                    if (CCF) {
                        const float vb = mb.add(a, j.npix + pix, t, cb.apply((float)((int)fb[f * fstride] - bgb), t,
                                                                             j.frametime, j.poly_order, a.basis));
                        db[(size_t)f * j.npix] = vb;
                    }
                }
            } else {
                for (int f = 0; f < n; f++) {
                    const int t = tb + f;
                    int wa = 0, wb = 0;
                    for (int k = 0; k < j.biny; k++)
                        for (int i = 0; i < j.binx; i++) {
                            wa += (int)fa[f * fstride + k * a.bw + i];
                            if (CCF) wb += (int)fb[f * fstride + k * a.bw + i];
                        }
                    const float va =
                        ma.add(a, pix, t, ca.apply((float)(wa - bga), t, j.frametime, j.poly_order, a.basis));
                    da[(size_t)f * j.npix] = va;
                    if (CCF) {
                        const float vb = mb.add(a, j.npix + pix, t,
                                                cb.apply((float)(wb - bgb), t, j.frametime, j.poly_order, a.basis));
                        db[(size_t)f * j.npix] = vb;
                    }
                }
            }
            if (tb + kStF >= min((seg + 1) * kSeg, t1)) {   // last box of the segment
                ma.store(a, pix, seg);
                if (CCF) mb.store(a, j.npix + pix, seg);
            }
        }
        __syncthreads();                                    // box `slot` is free
        if (tid == 0 && b + kStRing < nbox) {
            tma_load_box(&tmap, tiles + (size_t)slot * box, &full[slot], tx0, ry0,
                         j.first + t0 + (b + kStRing) * kStF, (uint32_t)box * 2);
            issued = b + kStRing + 1;
        }
    }
}

// Plain-load stream pass: grid (ceil(npix/128), nseg), one thread per
// (pixel, segment); the raw windows by 8-deep batches of loads.
template <int MODE, bool CCF>
__global__ void __launch_bounds__(128) stream_plain_kernel(StreamArgs a)
{
    const Job &j = a.j;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= j.npix) return;
    const int seg = blockIdx.y, t0 = seg * kSeg, t1 = min(t0 + kSeg, j.num);
    for (int tr = 0; tr < (CCF ? 2 : 1); tr++) {
        const int trace = tr ? j.npix + pix : pix;
        int x0, y0;
        trace_origin(j, trace, x0, y0);
        StreamCorr<MODE> c;
        c.load(a.bparams + (size_t)trace * kBleachStride, j.frametime);
        MonAcc m;
        m.init(a, t0);
        float *dst = tr ? a.s0b : a.s0a;
        const int bg = trace_bg(j, trace);
        for (int tb = t0; tb < t1; tb += 8) {
            if (((tb - t0) & (kStF - 1)) == 0) c.seed(tb, j.frametime);
            float v[8];
            window_values<8>(j, a.stack, x0, y0, tb, t1, bg, v);
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int t = tb + u;
                if (t >= t1) break;
                dst[(size_t)t * j.npix + pix] = m.add(a, trace, t, c.apply(v[u], t, j.frametime, j.poly_order, a.basis));
            }
        }
        m.store(a, trace, seg);
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct StreamPlan {
    int ok, nw, bw, bh, tiles_x;
    size_t smem;
};

static StreamPlan stream_plan(const Job &j, const void *stack)
{
    StreamPlan sp;
    memset(&sp, 0, sizeof(sp));
    if (j.input_float || ((uintptr_t)stack % 16) != 0 || (j.in_w % 8) != 0) return sp;   // TMA: 16-byte base and row stride
    for (int nw = 4; nw >= 1; nw >>= 1) {
        int bw = 7 + (32 * nw - 1) * j.pixbinx + j.binx + abs(j.cfx);
        bw = (bw + 7) & ~7;
        const int bh = j.biny + abs(j.cfy);
        const size_t smem = (size_t)kStRing * kStF * bw * bh * 2;
        if (bw > 256 || bh > 256 || smem > 100 * 1024) continue;
        sp.ok = 1;
        sp.nw = nw;
        sp.bw = bw;
        sp.bh = bh;
        sp.smem = smem;
        sp.tiles_x = (j.out_w + 32 * nw - 1) / (32 * nw);
        return sp;
    }
    return sp;
}

template <int MODE, bool CCF>
static cudaError_t launch_stream_t(const StreamArgs &a, const StreamPlan &sp, const CUtensorMap *map,
                                   cudaStream_t s)
{
    const Job &j = a.j;
    if (map) {
        auto kern = (j.binx == 1 && j.biny == 1) ? stream_tma_kernel<MODE, CCF, true> : stream_tma_kernel<MODE, CCF, false>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp.smem);
        if (e != cudaSuccess) return e;
        kern<<<dim3(sp.tiles_x * j.out_h, (a.nseg + kStSegs - 1) / kStSegs), 32 * sp.nw, sp.smem, s>>>(a, *map);
    } else {
        stream_plain_kernel<MODE, CCF><<<dim3((j.npix + 127) / 128, a.nseg), 128, 0, s>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_stream(const Job &j, const void *stack, const float *bparams, const float *basis,
                          const int *snap_pos, int nseg, float *s0, float2 *segtot, float2 *snap_part, int *segbad,
                          int *snap_bad, int *err, cudaStream_t s)
{
    StreamArgs a;
    memset(&a, 0, sizeof(a));
    a.j = j;
    a.stack = stack;
    a.bparams = bparams;
    a.basis = basis;
    a.snap_pos = snap_pos;
    a.nseg = nseg;
    a.s0a = s0;
    a.s0b = j.is_ccf ? s0 + (size_t)j.npix * j.num : s0;
    a.segtot = segtot;
    a.snap_part = snap_part;
    a.segbad = segbad;
    a.snap_bad = snap_bad;
    a.err = err;
    const StreamPlan sp = stream_plan(j, stack);
    CUtensorMap map;
    const CUtensorMap *mp = nullptr;
    PFN_cuTensorMapEncodeTiled_v12000 enc = sp.ok ? tensor_map_encoder() : nullptr;
    if (enc) {
        memset(&map, 0, sizeof(map));
        cuuint64_t dims[3] = {(cuuint64_t)j.in_w, (cuuint64_t)j.in_h, (cuuint64_t)(j.first + j.num)};
        cuuint64_t strides[2] = {(cuuint64_t)j.in_w * 2, (cuuint64_t)j.in_w * j.in_h * 2};
        cuuint32_t box[3] = {(cuuint32_t)sp.bw, (cuuint32_t)sp.bh, (cuuint32_t)kStF};
        cuuint32_t es[3] = {1, 1, 1};
        if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<void *>(stack), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS) {
            mp = &map;
            a.nw = sp.nw;
            a.tiles_x = sp.tiles_x;
            a.bw = sp.bw;
            a.bh = sp.bh;
        }
    }
    switch (j.bleach) {
    case IMFCS_BLEACH_SINGLE_EXP:
        return j.is_ccf ? launch_stream_t<1, true>(a, sp, mp, s) : launch_stream_t<1, false>(a, sp, mp, s);
    case IMFCS_BLEACH_DOUBLE_EXP:
        return j.is_ccf ? launch_stream_t<2, true>(a, sp, mp, s) : launch_stream_t<2, false>(a, sp, mp, s);
    case IMFCS_BLEACH_POLYNOMIAL:
        return j.is_ccf ? launch_stream_t<3, true>(a, sp, mp, s) : launch_stream_t<3, false>(a, sp, mp, s);
    default:
        return j.is_ccf ? launch_stream_t<0, true>(a, sp, mp, s) : launch_stream_t<0, false>(a, sp, mp, s);
    }
}

// ---------------------------------------------------------------------------
// N&B mode (isNBcalculation, agpufitjni.cu:5719-5720 and calcacf2b
// 5167-5180): only lag 1 is evaluated.  NBmean = the mean of the direct
// window's first num-1 samples, NBcov = <I(t) I'(t+1)> - NBmean <I'>, over
// the same num-1 products -- from the corrected, centred level-0 stream
// (shift-invariant) and the lag-1 monitors.  Grid (pixel blocks, frame
// segments); float-float segment sums combined by FP64 atomics.
// ---------------------------------------------------------------------------
constexpr int kNbSeg = 2048;

__global__ void nb_lag1_kernel(int npix, int num, const float *s0a, const float *s0b, double *sum)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const int t0 = blockIdx.y * kNbSeg, t1 = min(t0 + kNbSeg, num - 1);
    ff acc = {0.f, 0.f};
    for (int t = t0; t < t1; t++)
        ff_add(acc, __ldg(&s0a[(size_t)t * npix + pix]) * __ldg(&s0b[(size_t)(t + 1) * npix + pix]));
    atomicAdd(&sum[pix], ff_val(acc));
}

__global__ void nb_finalize_kernel(int npix, int chanum, int num, const float4 *mon, const double *sum,
                                   double *nb_mean, double *nb_cov)
{
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const float4 m = mon[(size_t)pix * chanum + 1];   // (a, b, dm, Dm) of lag 1
    const double n = (double)(num - 1);
    if (nb_mean) nb_mean[pix] = m.z;
    if (nb_cov) nb_cov[pix] = sum[pix] / n - (double)m.x * (double)m.y;
}

cudaError_t launch_nb_lag1(const Job &j, const float *s0, const float4 *mon, double *sum, double *nb_mean,
                           double *nb_cov, cudaStream_t s)
{
    const float *s0a = s0, *s0b = j.is_ccf ? s0 + (size_t)j.npix * j.num : s0;
    cudaError_t e = cudaMemsetAsync(sum, 0, sizeof(double) * j.npix, s);
    if (e != cudaSuccess) return e;
    dim3 grid((j.npix + 127) / 128, (j.num - 1 + kNbSeg - 1) / kNbSeg);
    nb_lag1_kernel<<<grid, 128, 0, s>>>(j.npix, j.num, s0a, s0b, sum);
    nb_finalize_kernel<<<(j.npix + 127) / 128, 128, 0, s>>>(j.npix, j.chanum, j.num, mon, sum, nb_mean, nb_cov);
    return cudaGetLastError();
}

}  // namespace imfcs
