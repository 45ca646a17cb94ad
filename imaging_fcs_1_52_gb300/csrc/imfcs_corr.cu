// imfcs_corr.cu -- streaming multi-tau correlator with blocked variance.
//
// Restates calculateCF (Imaging_FCS_1_52.java:9425-9648) for every output
// pixel at once.  One CTA owns 32 output pixels (one per lane) and streams
// the whole stack through shared memory in chunks of 128 frames:
//
//   stage   all warps compute the binned, background-subtracted,
//           bleach-corrected and centred value of each (pixel, frame) and
//           build the pairwise-binned levels 1..Q-1 (java:9467-9476),
//   correlate
//           warp 0: level 0, lags 0..8        warp 1: level 0, lags 9..16
//           warp 2: levels 1..Q-1 (lag delays 9..16 at each level)
//
// Products are grouped by their *direct* sample y: when the delayed samples
// y..y+16 are present, every lag's product d0[y]*d1[y+d] is accumulated.
// So the blocks of the blocked variance (2^(ind-k) products, java:9502-9511)
// end at the same y for every lag of a level, and the per-block sums of the
// direct and delayed samples come from two shared running sums plus the
// window "heads" (sum of the first d delayed samples of a block).  With the
// window means a, b known from the monitor pass, the centred block mean is
//   P_z = (A_z - b B_z - a D_z + L a b) / L
// exactly the Java blocked product (prod after binct pairwise means).
// Values are FP32 centred on the pixel's mean; block sums are exact-order FP32,
// totals are float-float.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "imfcs_corr.cuh"
#include "imfcs_tma.cuh"

namespace imfcs {

constexpr int kCorrThreads = 128;

// Block end for the lags [lagbase, lagbase+nl) of one level (out of line:
// it runs once per 2^(ind-k) direct samples).  acc: the lags' block sums of
// products; head_sm: this level's heads (stride 32); wsm: delayed samples
// y+1..y+16 in shared memory (stride 32); z: block number.
__device__ __noinline__ void block_end(const Job &j, const CorrOut &o, const float4 *mon, int pix,
                                       int lagbase, int del0, int nl, float *acc, float B0,
                                       float B1, float *head_sm, const float *wsm, int z, int L,
                                       int pnum)
{
    float nh[kP + 1];
    nh[0] = 0.f;
    for (int d = 1; d <= kP; d++) nh[d] = nh[d - 1] + wsm[(d - 1) * 32];
    const float invL = 1.f / (float)L;
    for (int l = 0; l < nl; l++) {
        const int d = del0 + l, lag = lagbase + l;
        const float4 m = mon[(size_t)pix * j.chanum + lag];
        const float a = m.x, b = m.y;
        float D = B1 - head_sm[d * 32] + nh[d];
        float P = (acc[l] - b * B0 - a * D + (float)L * a * b) * invL;
        float &ahi = stat_ref(o.stats, j.npix, lag, 0, pix);
        float &alo = stat_ref(o.stats, j.npix, lag, 1, pix);
        ff t = {ahi, alo};
        ff_add(t, acc[l]);
        ahi = t.hi;
        alo = t.lo;
        if (z < pnum) {
            float &r = stat_ref(o.stats, j.npix, lag, 4, pix);
            if (z == 0) r = P;
            float dv = P - r;
            stat_ref(o.stats, j.npix, lag, 2, pix) += dv;
            stat_ref(o.stats, j.npix, lag, 3, pix) += dv * dv;
            if (o.gls && lag >= 1) o.bprod[((size_t)pix * (j.chanum - 1) + (lag - 1)) * o.pnum_stride + z] = P;
        }
        acc[l] = 0.f;
    }
    for (int d = 0; d <= kP; d++) head_sm[d * 32] = nh[d];
}

// Heads of the first block: sums of the first d delayed samples.
__device__ __noinline__ void block_head_init(float *head_sm, const float *wsm)
{
    float h = 0.f;
    head_sm[0] = 0.f;
    for (int d = 1; d <= kP; d++) { h += wsm[(d - 1) * 32]; head_sm[d * 32] = h; }
}

// One branch-free group of 16 direct samples (positions i0..i0+15) with the
// delayed samples in a register ring: w[(PH + j + d) & 31] holds position
// i0 + j + d.  Loads the delayed samples of the next group on the way.
template <int NL, int DEL0, int PH>
__device__ __forceinline__ void group16(const float *buf0, const float *buf1, int i0, float (&w)[32],
                                        float *acc, float &B0, float &B1)
{
#pragma unroll
    for (int jj = 0; jj < 16; jj++) {
        const int i = i0 + jj;
        w[(PH + jj + kP) & 31] = buf1[(i + kP) * 32];
        const float x0 = buf0[i * 32];
#pragma unroll
        for (int l = 0; l < NL; l++) acc[l] = fmaf(x0, w[(PH + jj + DEL0 + l) & 31], acc[l]);
        B0 += x0;
        B1 += w[(PH + jj) & 31];
    }
}

// Generic per-sample path (range checks, first-block heads, block ends at
// any sample); used where a group is not entirely regular.
template <int NL, int DEL0>
__device__ __forceinline__ void samples_slow(const Job &j, const CorrOut &o, const float4 *mon, int pix,
                                             int lagbase, const float *buf0, const float *buf1, int i0,
                                             int i1, int ybeg, int numbin, int L, int pnum, float *acc,
                                             float &B0, float &B1, float *head_sm)
{
    for (int i = i0; i < i1; i++) {
        const int y = ybeg + i;
        if (y < 0 || y >= numbin) continue;
        const float x0 = buf0[i * 32];
        if (y == 0) block_head_init(head_sm, buf1 + i * 32);
#pragma unroll
        for (int l = 0; l < NL; l++) acc[l] = fmaf(x0, buf1[(i + DEL0 + l) * 32], acc[l]);
        B0 += x0;
        B1 += buf1[i * 32];
        if ((y & (L - 1)) == L - 1) {
            float tmp[NL];
#pragma unroll
            for (int l = 0; l < NL; l++) tmp[l] = acc[l];
            block_end(j, o, mon, pix, lagbase, DEL0, NL, tmp, B0, B1, head_sm, buf1 + (i + 1) * 32, y / L, L,
                      pnum);
#pragma unroll
            for (int l = 0; l < NL; l++) acc[l] = 0.f;
            B0 = 0.f;
            B1 = 0.f;
        }
    }
}

// One group of 16 samples at ring phase PH: fast path when, for every lane,
// the group lies inside [1, numbin) and blocks are at least 16 long (then a
// block can only end on the group's last sample, y = 16m + 15).
template <int NL, int DEL0, int PH>
__device__ __forceinline__ void group_step(const Job &j, const CorrOut &o, const float4 *mon, int pix,
                                           bool valid, int lagbase, const float *buf0, const float *buf1,
                                           int i0, int ybeg, int numbin, int L, int pnum, float (&w)[32],
                                           float *acc, float &B0, float &B1, float *head_sm)
{
    // every lane of the warp takes part in the vote; lanes without a pixel
    // (last CTA) vote "fast", compute on zeros and write nothing
    const int y0 = ybeg + i0, y1 = y0 + 15;
    const bool fast = !valid || ((y0 >= 1) && (y1 < numbin) && (L >= 16));
    if (__all_sync(0xffffffffu, fast)) {
        group16<NL, DEL0, PH>(buf0, buf1, i0, w, acc, B0, B1);
        if (valid && (y1 & (L - 1)) == L - 1) {
            float tmp[NL];
#pragma unroll
            for (int l = 0; l < NL; l++) tmp[l] = acc[l];
            block_end(j, o, mon, pix, lagbase, DEL0, NL, tmp, B0, B1, head_sm, buf1 + (i0 + 16) * 32, y1 / L,
                      L, pnum);
#pragma unroll
            for (int l = 0; l < NL; l++) acc[l] = 0.f;
            B0 = 0.f;
            B1 = 0.f;
        }
    } else {
        if (valid)
            samples_slow<NL, DEL0>(j, o, mon, pix, lagbase, buf0, buf1, i0, i0 + 16, ybeg, numbin, L, pnum,
                                   acc, B0, B1, head_sm);
        // keep the ring valid for the next group (positions i0+16..i0+31)
#pragma unroll
        for (int jj = 0; jj < 16; jj++) w[(PH + 16 + jj) & 31] = buf1[(i0 + 16 + jj) * 32];
    }
}

// Process the direct samples of one level held in shared memory.
// buf0/buf1: level buffers (already offset by lane), [kHist + nnew] x 32;
// position i holds sample s_begin - kHist + i.  Direct samples are
// positions [0, nnew).  GROUPED requires nnew % 16 == 0 (s_begin is then a
// multiple of 16, so groups start at y = 16m).
template <int NL, int DEL0, bool GROUPED>
__device__ __forceinline__ void correlate_level(const Job &j, const CorrOut &o, const float4 *mon,
                                                int pix, bool valid, int lagbase, const float *buf0,
                                                const float *buf1, int nnew, int s_begin, int numbin,
                                                int L, int pnum, float *acc, float &B0, float &B1,
                                                float *head_sm)
{
    const int ybeg = s_begin - kHist;
    if (ybeg >= numbin || ybeg + nnew <= 0) return;
    if (GROUPED) {
        float w[32];
#pragma unroll
        for (int d = 0; d < kP; d++) w[d] = buf1[d * 32];
        for (int g = 0; g < nnew; g += 32) {
            group_step<NL, DEL0, 0>(j, o, mon, pix, valid, lagbase, buf0, buf1, g, ybeg, numbin, L, pnum, w, acc,
                                    B0, B1, head_sm);
            if (g + 16 < nnew)
                group_step<NL, DEL0, 16>(j, o, mon, pix, valid, lagbase, buf0, buf1, g + 16, ybeg, numbin, L, pnum,
                                         w, acc, B0, B1, head_sm);
        }
    } else if (valid) {
        samples_slow<NL, DEL0>(j, o, mon, pix, lagbase, buf0, buf1, 0, nnew, ybeg, numbin, L, pnum, acc, B0,
                               B1, head_sm);
    }
}

// Shared-memory layout: per level k a buffer of (kHist + kChunk/2^k) x 32
// floats for the direct trace, and (CCF only) one for the delayed trace.
__host__ __device__ inline int level_cap(int k) { return kHist + (kChunk >> k); }
__host__ __device__ inline int level_off(int k)
{
    int o = 0;
    for (int i = 0; i < k; i++) o += level_cap(i) * 32;
    return o;
}

// Per-level persistent state of the binned-level warps in shared memory:
// acc[8], B0, B1, head[17] per level and lane.  Level 0 keeps acc, B0, B1 in
// registers of warps 0 and 1; each of those warps has its own head[17].
constexpr int kLvlState = 8 + 2 + kP + 1;
constexpr int kHead0 = 2 * (kP + 1);

__host__ __device__ inline size_t corr_smem_floats_dev(int q, bool ccf)
{
    return (size_t)(ccf ? 2 : 1) * level_off(q) + (size_t)q * kLvlState * 32 + kHead0 * 32;
}

// ---------------------------------------------------------------------------
// TMA staging of the raw uint16 frames: one box [kChunk][BH][BW] per chunk,
// loaded by one thread while the CTA correlates the previous chunk.  Waits
// are bounded: on a timeout the CTA records an error and leaves.
// ---------------------------------------------------------------------------
// Window value of a trace from the staged raw tile (frame fr of the chunk).
__device__ __forceinline__ float tile_value(const Job &j, const uint16_t *tile, int BW, int BH, int fr, int xr, int yr,
                                            int bg)
{
    const uint16_t *f = tile + (size_t)fr * BH * BW;
    int acc = 0;
    for (int k = 0; k < j.biny; k++)
        for (int i = 0; i < j.binx; i++) acc += (int)f[(yr + k) * BW + xr + i];
    return (float)(acc - bg);
}

struct TmaGeom {
    int use_tma;       // raw frames staged by TMA
    int bw, bh;        // box width / height (elements); box depth is kChunk
};

template <bool CCF>
__global__ void __launch_bounds__(kCorrThreads) corr_kernel(Job j, const LagInfo *li_g, const void *stack,
                                                            const float *bparams, const float *basis,
                                                            const float4 *mon, const int *blk_ind, CorrOut o,
                                                            TmaGeom tg, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) float smem[];
    const int nlev = j.q;                 // levels 0..q-1
    const int buf_floats = level_off(nlev);
    float *buf0 = smem;
    float *buf1 = CCF ? smem + buf_floats : smem;
    float *lvl_state = smem + (CCF ? 2 : 1) * buf_floats;   // [level][kLvlState][32]
    float *head0_sm = lvl_state + nlev * kLvlState * 32;     // [warp 0/1][kP+1][32]
    // [kChunk][bh][bw] raw frames (TMA destination, 128-byte aligned)
    uint16_t *raw;
    {
        const uint32_t base = smem_u32(smem);
        const uint32_t want = (base + (uint32_t)(corr_smem_floats_dev(nlev, CCF) * sizeof(float)) + 127u) & ~127u;
        raw = (uint16_t *)((char *)smem + (want - base));
    }
    __shared__ float sh_basis[kChunk * (kMaxPoly + 1)];
    __shared__ int sh_numbin[kMaxLevels];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ int sh_fail;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // CTA = a segment of 32 pixels of one output row
    const int tiles_per_row = (j.out_w + 31) / 32;
    const int oy = blockIdx.x / tiles_per_row, seg = blockIdx.x % tiles_per_row;
    const int ox = seg * 32 + lane;
    const bool pvalid = ox < j.out_w && oy < j.out_h;
    const int pix = oy * j.out_w + ox;
    const int pixc = pvalid ? pix : oy * j.out_w + seg * 32;
    if (tid < kMaxLevels) sh_numbin[tid] = tid < nlev ? li_g->numbin[tid] : 0;
    if (tid == 0) sh_fail = 0;

    // trace origins and bleach parameters of this lane's pixel
    int xa, ya, xb, yb;
    trace_origin(j, pixc, xa, ya);
    const int trb = CCF ? j.npix + pixc : pixc;
    trace_origin(j, trb, xb, yb);
    const int bga = trace_bg(j, pixc), bgb = trace_bg(j, trb);
    // tile origin (x rounded down to 8 elements for TMA alignment)
    const int xt0 = (j.map_x0 + seg * 32) * j.pixbinx;
    const int yt0 = (j.map_y0 + oy) * j.pixbiny;
    const int tx0 = (min(xt0, xt0 + j.cfx)) & ~7;
    const int ty0 = min(yt0, yt0 + j.cfy);
    float bpa[kBleachStride], bpb[kBleachStride];
#pragma unroll
    for (int i = 0; i < kBleachStride; i++) {
        bpa[i] = __ldg(&bparams[(size_t)pixc * kBleachStride + i]);
        bpb[i] = CCF ? __ldg(&bparams[(size_t)trb * kBleachStride + i]) : bpa[i];
    }
    const int ind = pvalid ? blk_ind[pixc] : (j.q - 1);
    const int pnum = li_g->pnum_by_ind[ind];

    // zero the block statistics of this lane's lags
    if (pvalid) {
        int lag_lo, lag_hi;
        if (warp == 0) { lag_lo = 0; lag_hi = 9; }
        else if (warp == 1) { lag_lo = 9; lag_hi = 17; }
        else if (warp == 2) { lag_lo = 17; lag_hi = min(25, j.chanum); }
        else { lag_lo = 25; lag_hi = j.chanum; }
        for (int lag = lag_lo; lag < lag_hi; lag++)
            for (int s = 0; s < kStatN; s++) stat_ref(o.stats, j.npix, lag, s, pix) = 0.f;
    }
    // zero level state and history
    for (int i = tid; i < nlev * kLvlState * 32; i += kCorrThreads) lvl_state[i] = 0.f;
    for (int k = 0; k < nlev; k++)
        for (int i = tid; i < kHist * 32; i += kCorrThreads) {
            buf0[level_off(k) + i] = 0.f;
            if (CCF) buf1[level_off(k) + i] = 0.f;
        }
    float acc0[9], B00 = 0.f, B10 = 0.f;
#pragma unroll
    for (int l = 0; l < 9; l++) acc0[l] = 0.f;
    for (int i = tid; i < kHead0 * 32; i += kCorrThreads) head0_sm[i] = 0.f;

    const int order1 = j.poly_order + 1;
    const int numbin_last = li_g->numbin[nlev - 1];
    const int top_n = kChunk >> (nlev - 1);
    int nchunks = (numbin_last + kHist + top_n - 1) / top_n;
    const int nchunk0 = (j.num + kChunk - 1) / kChunk;
    if (nchunks < nchunk0 + 1) nchunks = nchunk0 + 1;
    const uint32_t box_bytes = (uint32_t)kChunk * tg.bh * tg.bw * 2u;

    if (tg.use_tma && tid == 0) {
        mbar_init(&mbar, 1);
        tma_load_box(&tmap, raw, &mbar, tx0, ty0, j.first, box_bytes);
    }
    // basis table of chunk 0
    if (j.bleach == IMFCS_BLEACH_POLYNOMIAL)
        for (int i = tid; i < kChunk * order1; i += kCorrThreads)
            sh_basis[i] = (i / order1) < j.num ? __ldg(&basis[i]) : 0.f;
    __syncthreads();

    for (int c = 0; c < nchunks; c++) {
        const int f0 = c * kChunk;
        // ---- stage: level-0 values (binned, background, bleach, centred) ----
        if (f0 < j.num) {
            if (tg.use_tma) {
                bool ok = mbar_wait(&mbar, (uint32_t)(c & 1));
                if (!ok) sh_fail = 1;
            }
            for (int fr = warp; fr < kChunk; fr += kCorrThreads / 32) {
                const int f = f0 + fr;
                float va = 0.f, vb = 0.f;
                if (f < j.num && pvalid) {
                    float t = frame_time(j, f);
                    const float *bs = sh_basis + fr * order1;
                    va = tg.use_tma ? tile_value(j, raw, tg.bw, tg.bh, fr, xa - tx0, ya - ty0, bga)
                                    : window_value(j, stack, xa, ya, f, bga);
                    if (j.bleach != IMFCS_BLEACH_NONE && bpa[11] != 0.f)
                        va = bleach_correct(va, bleach_f(bpa, j.bleach, j.poly_order, t, bs), bpa[9], bpa[10]);
                    va -= bpa[12];
                    if (CCF) {
                        vb = tg.use_tma ? tile_value(j, raw, tg.bw, tg.bh, fr, xb - tx0, yb - ty0, bgb)
                                        : window_value(j, stack, xb, yb, f, bgb);
                        if (j.bleach != IMFCS_BLEACH_NONE && bpb[11] != 0.f)
                            vb = bleach_correct(vb, bleach_f(bpb, j.bleach, j.poly_order, t, bs), bpb[9], bpb[10]);
                        vb -= bpb[12];
                    }
                }
                // non-finite frames enter as 0: the monitors make exactly the
                // lags whose windows hold one non-finite
                buf0[(kHist + fr) * 32 + lane] = isfinite(va) ? va : 0.f;
                if (CCF) buf1[(kHist + fr) * 32 + lane] = isfinite(vb) ? vb : 0.f;
            }
        } else {
            for (int i = tid; i < kChunk * 32; i += kCorrThreads) {
                buf0[kHist * 32 + i] = 0.f;
                if (CCF) buf1[kHist * 32 + i] = 0.f;
            }
        }
        __syncthreads();
        if (sh_fail) {
            if (tid == 0 && o.err) atomicExch(o.err, 1);
            return;   // uniform: every thread read sh_fail after the barrier
        }
        // the raw tile is free again: prefetch the next chunk's frames
        if (tg.use_tma && tid == 0 && f0 + kChunk < j.num)
            tma_load_box(&tmap, raw, &mbar, tx0, ty0, j.first + f0 + kChunk, box_bytes);

        // ---- correlate (all lanes take part, so warp votes see full warps) ----
        const int numbin0 = sh_numbin[0];
        if (warp < 2) {
            const int L = 1 << ind;
            float *hs = head0_sm + warp * (kP + 1) * 32 + lane;
            if (warp == 0)
                correlate_level<9, 0, true>(j, o, mon, pixc, pvalid, 0, buf0 + lane, buf1 + lane, kChunk, f0,
                                            numbin0, L, pnum, acc0, B00, B10, hs);
            else
                correlate_level<8, 9, true>(j, o, mon, pixc, pvalid, 9, buf0 + lane, buf1 + lane, kChunk, f0,
                                            numbin0, L, pnum, acc0, B00, B10, hs);
        } else {
            if (warp == 2) {
                // build the binned levels 1..q-1 by pairwise sums (java:9467-9476)
                for (int k = 1; k < nlev; k++) {
                    const int nk = kChunk >> k, sb = c * nk, nb = sh_numbin[k];
                    for (int s = 0; s < nk; s++) {
                        const bool v = (sb + s) < nb;
                        const float *p0 = buf0 + level_off(k - 1) + (kHist + 2 * s) * 32 + lane;
                        buf0[level_off(k) + (kHist + s) * 32 + lane] = v ? p0[0] + p0[32] : 0.f;
                        if (CCF) {
                            const float *p1 = buf1 + level_off(k - 1) + (kHist + 2 * s) * 32 + lane;
                            buf1[level_off(k) + (kHist + s) * 32 + lane] = v ? p1[0] + p1[32] : 0.f;
                        }
                    }
                    __syncwarp();
                }
                asm volatile("bar.arrive 1, 64;" ::: "memory");
            } else {
                asm volatile("bar.sync 1, 64;" ::: "memory");
            }
            // warp 2: level 1; warp 3: levels 2..q-1
            const int kb = (warp == 2) ? 1 : 2, ke = (warp == 2) ? min(2, nlev) : nlev;
            for (int k = kb; k < ke; k++) {
                const int nk = kChunk >> k;
                const int numbin = sh_numbin[k];
                const int sb = c * nk;
                if (sb - kHist >= numbin) continue;
                float *st = lvl_state + (size_t)k * kLvlState * 32;
                float acc[8], B0, B1;
#pragma unroll
                for (int l = 0; l < 8; l++) acc[l] = st[l * 32 + lane];
                B0 = st[8 * 32 + lane];
                B1 = st[9 * 32 + lane];
                float *hs = st + 10 * 32 + lane;
                const int L = 1 << (ind - k);
                const int lagbase = (kP + 1) + (k - 1) * 8;
                if (nk >= 16)
                    correlate_level<8, 9, true>(j, o, mon, pixc, pvalid, lagbase, buf0 + level_off(k) + lane,
                                                buf1 + level_off(k) + lane, nk, sb, numbin, L, pnum, acc, B0, B1, hs);
                else
                    correlate_level<8, 9, false>(j, o, mon, pixc, pvalid, lagbase, buf0 + level_off(k) + lane,
                                                 buf1 + level_off(k) + lane, nk, sb, numbin, L, pnum, acc, B0, B1, hs);
#pragma unroll
                for (int l = 0; l < 8; l++) st[l * 32 + lane] = acc[l];
                st[8 * 32 + lane] = B0;
                st[9 * 32 + lane] = B1;
            }
        }
        __syncthreads();
        // ---- shift history: the last kHist samples of each level to the
        // front.  Levels with at least kHist new samples copy in place (no
        // overlap); the others (at most 4: kChunk/2^k < kHist) overlap source
        // and destination and go through registers.
        float hv0[4][4], hv1[4][4];
        for (int k = 0; k < nlev; k++) {
            const int nk = kChunk >> k;
            if (nk >= kHist) {
                for (int i = tid; i < kHist * 32; i += kCorrThreads) {
                    buf0[level_off(k) + i] = buf0[level_off(k) + nk * 32 + i];
                    if (CCF) buf1[level_off(k) + i] = buf1[level_off(k) + nk * 32 + i];
                }
            }
        }
        const int ksmall = 5;   // kChunk >> k < kHist for k >= 4 (kChunk = 128, kHist = 16)
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const int k = ksmall - 1 + m;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int i = tid + r * kCorrThreads;
                hv0[m][r] = (k < nlev) ? buf0[level_off(k) + (kChunk >> k) * 32 + i] : 0.f;
                hv1[m][r] = (CCF && k < nlev) ? buf1[level_off(k) + (kChunk >> k) * 32 + i] : 0.f;
            }
        }
        __syncthreads();
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const int k = ksmall - 1 + m;
            if (k >= nlev) continue;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int i = tid + r * kCorrThreads;
                buf0[level_off(k) + i] = hv0[m][r];
                if (CCF) buf1[level_off(k) + i] = hv1[m][r];
            }
        }
        if (j.bleach == IMFCS_BLEACH_POLYNOMIAL && f0 + kChunk < j.num)
            for (int i = tid; i < kChunk * order1; i += kCorrThreads)
                sh_basis[i] = (f0 + kChunk + i / order1) < j.num ? __ldg(&basis[(size_t)(f0 + kChunk) * order1 + i]) : 0.f;
        __syncthreads();
    }

    // ---- finalise: remaining partial block into the totals, outputs ----
    if (!pvalid) return;
    int lag_lo, lag_hi;
    if (warp == 0) lag_lo = 0, lag_hi = 9;
    else if (warp == 1) lag_lo = 9, lag_hi = 17;
    else if (warp == 2) lag_lo = 17, lag_hi = min(25, j.chanum);
    else lag_lo = 25, lag_hi = j.chanum;
    for (int lag = lag_lo; lag < lag_hi; lag++) {
        float rem;
        if (warp < 2) {
            rem = 0.f;
#pragma unroll
            for (int l = 0; l < 9; l++)
                if (l == lag - lag_lo) rem = acc0[l];
        } else {
            int k = 1 + (lag - 17) / 8, l = (lag - 17) % 8;
            rem = lvl_state[(size_t)k * kLvlState * 32 + l * 32 + lane];
        }
        float &ahi = stat_ref(o.stats, j.npix, lag, 0, pix);
        float &alo = stat_ref(o.stats, j.npix, lag, 1, pix);
        ff t = {ahi, alo};
        ff_add(t, rem);
        const double A = ff_val(t);
        const double S1 = stat_ref(o.stats, j.npix, lag, 2, pix);
        const double S2 = stat_ref(o.stats, j.npix, lag, 3, pix);
        const float4 m = mon[(size_t)pix * j.chanum + lag];
        const double n = li_g->prodnum[lag];
        const double dmDm = (double)m.z * (double)m.w;
        const double sumprod = A - n * (double)m.x * (double)m.y;
        const double corav = sumprod / (n * dmDm);
        const double pn = pnum;
        const double bv = (S2 / pn - (S1 / pn) * (S1 / pn)) / ((pn - 1) * dmDm * dmDm);
        double acf = corav;
        if (o.gls) {
            const double r = stat_ref(o.stats, j.npix, lag, 4, pix);
            acf = (lag == 0) ? 0.0 : (S1 + pn * r) / (pn * dmDm);   // mcov (java:9526-9531)
        }
        if (o.acf) o.acf[(size_t)pix * j.chanum + lag] = acf;
        if (o.var) o.var[(size_t)pix * j.chanum + lag] = bv;
        if (o.sd) o.sd[(size_t)pix * j.chanum + lag] = sqrt(bv);
        if (lag == 1) {
            if (o.nb_mean) o.nb_mean[pix] = m.z;
            if (o.nb_cov) o.nb_cov[pix] = sumprod / n;
        }
    }
}

template __global__ void corr_kernel<false>(Job, const LagInfo *, const void *, const float *, const float *,
                                            const float4 *, const int *, CorrOut, TmaGeom,
                                            const __grid_constant__ CUtensorMap);
template __global__ void corr_kernel<true>(Job, const LagInfo *, const void *, const float *, const float *,
                                           const float4 *, const int *, CorrOut, TmaGeom,
                                           const __grid_constant__ CUtensorMap);

// ---------------------------------------------------------------------------
// Host side: shared memory size, TMA geometry and tensor map, launch.  Jobs
// with Q >= 5 run the per-pixel kernel of imfcs_corr2.cu; this CTA-tiled
// kernel covers the rest (blocks shorter than 16 samples).
// ---------------------------------------------------------------------------
bool corr2_supported(const Job &j);
bool corrg_supported(const Job &j);
cudaError_t launch_corrg(const Job &j, const LagInfo *li, const float *s0, const float4 *mon, const int *blk_ind,
                         const CorrOut &o, cudaStream_t stream);
cudaError_t launch_corr2(const Job &j, const LagInfo *li, const float *s0, const float4 *mon, const int *blk_ind,
                         const CorrOut &o, float *streams, cudaStream_t stream);

size_t corr_smem_bytes(int q, bool ccf) { return corr_smem_floats_dev(q, ccf) * sizeof(float); }

// TMA box over the raw stack that covers every window of a 32-pixel row
// segment (x rounded down to 8 elements = 16 bytes).
static TmaGeom tma_geometry(const Job &j, const void *stack)
{
    TmaGeom g{0, 0, 0};
    if (j.input_float) return g;
    if ((j.in_w % 8) != 0 || ((uintptr_t)stack % 16) != 0) return g;
    int bw = 31 * j.pixbinx + j.binx + abs(j.cfx) + 7;
    bw = (bw + 7) & ~7;
    int bh = j.biny + abs(j.cfy);
    if (bw > 256 || bh > 256) return g;
    size_t bytes = (size_t)kChunk * bw * bh * 2;
    if (bytes > 40 * 1024) return g;
    g.use_tma = 1;
    g.bw = bw;
    g.bh = bh;
    return g;
}

static bool encode_stack_map(const Job &j, const void *stack, const TmaGeom &g, CUtensorMap *map)
{
    PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
    if (!fn) return false;
    const int frames_total = j.first + j.num;
    cuuint64_t dims[3] = {(cuuint64_t)j.in_w, (cuuint64_t)j.in_h, (cuuint64_t)frames_total};
    cuuint64_t strides[2] = {(cuuint64_t)j.in_w * 2, (cuuint64_t)j.in_w * j.in_h * 2};
    cuuint32_t box[3] = {(cuuint32_t)g.bw, (cuuint32_t)g.bh, (cuuint32_t)kChunk};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<void *>(stack), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

cudaError_t launch_corr(const Job &j, const LagInfo *li, const void *stack, const float *bparams,
                        const float *basis, const float *s0, const float4 *mon, const int *blk_ind, double *acf,
                        double *var, double *sd, double *nb_mean, double *nb_cov, float *bprod,
                        int pnum_stride, float *stats, float *streams, int gls, int *err,
                        cudaStream_t stream)
{
    CorrOut o;
    o.acf = acf; o.var = var; o.sd = sd; o.nb_mean = nb_mean; o.nb_cov = nb_cov;
    o.bprod = bprod; o.pnum_stride = pnum_stride; o.stats = stats; o.gls = gls; o.err = err;
    if (corr2_supported(j)) return launch_corr2(j, li, s0, mon, blk_ind, o, streams, stream);
    if (corrg_supported(j)) return launch_corrg(j, li, s0, mon, blk_ind, o, stream);
    TmaGeom g = tma_geometry(j, stack);
    CUtensorMap map;
    memset(&map, 0, sizeof(map));
    if (g.use_tma && !encode_stack_map(j, stack, g, &map)) g.use_tma = 0;
    size_t smem = corr_smem_bytes(j.q, j.is_ccf);
    if (g.use_tma) smem += 128 + (size_t)kChunk * g.bw * g.bh * 2;   // 128: alignment slack
    const int tiles_per_row = (j.out_w + 31) / 32;
    dim3 grid(tiles_per_row * j.out_h);
    if (j.is_ccf) {
        cudaFuncSetAttribute(corr_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        corr_kernel<true><<<grid, kCorrThreads, smem, stream>>>(j, li, stack, bparams, basis, mon, blk_ind, o, g, map);
    } else {
        cudaFuncSetAttribute(corr_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        corr_kernel<false><<<grid, kCorrThreads, smem, stream>>>(j, li, stack, bparams, basis, mon, blk_ind, o, g, map);
    }
    return cudaGetLastError();
}

}  // namespace imfcs
