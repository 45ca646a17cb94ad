// imfcs_corr2.cu -- multi-tau correlator with blocked variance as a chain of
// streaming kernels, no block-wide synchronisation.
//
// Restates calculateCF (Imaging_FCS_1_52.java:9425-9648) with the same
// per-lag block statistics and outputs as corr_kernel:
//
//   values    the binned, background-subtracted, bleach-corrected and
//             centred value of every (trace, frame) is written once as FP32,
//             frame-major ([t][pixel]): the level-0 sample stream s0;
//   pair k    one thread per (pixel, frame segment) streams the level-k
//             samples and correlates levels k and k+1 (lags 0..16 at level 0,
//             delays 9..16 above) in registers: rings of the last 32 samples
//             whose positions are compile-time constants inside a 64-sample
//             unrolled step; it writes the level-(k+2) samples (pair sums of
//             its level-(k+1) samples) for the next kernel;
//   tail      levels k0..Q-1 (blocks possibly one sample long): one level per
//             thread, samples built from the level-k0 stream, block
//             statistics in registers;
//   finalise  per (pixel, lag): segments combined in FP64, outputs.
//
// Products are grouped by their direct sample y (processed when the delayed
// samples y..y+16 are present), so the blocks of the blocked variance
// (2^(ind-k) products, java:9502-9511) end at the same y for every lag of a
// level.  With the window means a, b of the centred samples from the monitor
// pass, the blocked product of block z is
//   P_z = (A_z - b B_z - a D_z + L a b) / L
// (A_z: sum of products, B_z: sum of direct samples, D_z: sum of the delayed
// samples y+d over the block, from the block's running sum and the "heads",
// the sums of the first d delayed samples of a block).  Frame segments are
// multiples of every pixel's block length (2^ind frames), so no block spans
// two threads; each segment keeps its own statistics.
#include "imfcs_corr.cuh"

namespace imfcs {

constexpr int kC2Threads = 64;       // pixels per CTA unless the tile says 32
constexpr int kMaxSegExtra = 4;
constexpr int kHeadFields = (kP + 1) + 8;                   // first-level heads d = 0..16, second-level d = 9..16

// Arguments shared by the pair, tail and finalise kernels.
struct C2Args {
    CorrOut o;
    const float4 *mon;        // [pix][chanum] (a, b, dm, Dm)
    const int *blk_ind;       // [pix]
    const LagInfo *li;
    int npix, chanum, p, q, num;
    int numbin[kMaxLevels];
    int seg_log[kMaxLevels];  // frame segment (log2) of the kernel owning each level
    size_t stat_stride;       // floats per segment in o.stats
};

// Per-thread context.
struct C2Ctx {
    float *stats;             // this segment's statistics
    const float4 *mon;        // this pixel's monitors
    float *bprod;
    int npix, pix, chanum, pnum_stride, gls;
    int ind, pnum, zfirst;
    bool valid;               // false: a lane without a pixel (computes, writes nothing)
    // where the block statistics of this (pixel, segment) live: the global
    // array (stride npix) or a shared-memory copy (stride = threads) that the
    // caller writes back; and (optional) the lags' monitors (a, b) in shared
    // memory with stride smon_stride, both from lag lag0 on
    float *sst;
    int sst_stride;
    const float2 *smon;
    int smon_stride;
    int lag0;
    __device__ __forceinline__ float &stat(int lag, int s) const
    {
        return sst[(size_t)((lag - lag0) * kStatN + s) * sst_stride];
    }
    __device__ __forceinline__ float2 monitor(int lag) const
    {
        if (smon) return smon[(lag - lag0) * smon_stride];
        const float4 m = __ldg(&mon[lag]);
        return make_float2(m.x, m.y);
    }
};

// One block end of one lag: total, blocked product and its statistics.
__device__ __forceinline__ void c2_block_stat(const C2Ctx &c, int lag, float A, float B0, float D, int L, int z)
{
    if (!c.valid) return;
    const float2 m = c.monitor(lag);
    const float a = m.x, b = m.y;
    const float P = (A - b * B0 - a * D + (float)L * a * b) / (float)L;
    float &ahi = c.stat(lag, 0);
    float &alo = c.stat(lag, 1);
    ff t = {ahi, alo};
    ff_add(t, A);
    ahi = t.hi;
    alo = t.lo;
    if (z < c.pnum) {
        float &r = c.stat(lag, 4);
        if (z == c.zfirst) r = P;      // per-segment shift of the block statistics
        const float dv = P - r;
        c.stat(lag, 2) += dv;
        c.stat(lag, 3) += dv * dv;
        if (c.gls && lag >= 1) c.bprod[((size_t)c.pix * (c.chanum - 1) + (lag - 1)) * c.pnum_stride + z] = P;
    }
}

__device__ __forceinline__ void c2_add_total(const C2Ctx &c, int lag, float A)
{
    if (!c.valid) return;
    float &ahi = c.stat(lag, 0);
    float &alo = c.stat(lag, 1);
    ff t = {ahi, alo};
    ff_add(t, A);
    ahi = t.hi;
    alo = t.lo;
}

__device__ __forceinline__ void c2_ctx(C2Ctx &c, const C2Args &a, int pix, int seg, int k)
{
    c.valid = pix < a.npix;
    if (!c.valid) pix = a.npix - 1;   // reads stay in bounds; writes are masked
    c.stats = a.o.stats + (size_t)seg * a.stat_stride;
    c.mon = a.mon + (size_t)pix * a.chanum;
    c.bprod = a.o.bprod;
    c.npix = a.npix;
    c.pix = pix;
    c.chanum = a.chanum;
    c.pnum_stride = a.o.pnum_stride;
    c.gls = a.o.gls;
    c.ind = a.blk_ind[pix];
    c.pnum = a.li->pnum_by_ind[c.ind];
    c.zfirst = (seg << a.seg_log[k]) >> c.ind;
    c.sst = c.stats + pix;
    c.sst_stride = a.npix;
    c.smon = nullptr;
    c.smon_stride = 0;
    c.lag0 = 0;
}

// ---------------------------------------------------------------------------
// Pair kernel: levels k (first) and k+1 (second) of one (pixel, segment).
// FIRST17: the first level is level 0 (lags 0..16); otherwise its lags are
// delays 9..16.  TWO: the second level exists (k+1 < Q).
// ---------------------------------------------------------------------------
template <bool FIRST17>
struct PairReg {
    static constexpr int NF = FIRST17 ? kP + 1 : 8;   // first-level lags
    static constexpr int DF = FIRST17 ? 0 : 9;        // first-level delay of lag 0
    float wB[32], wA[32];      // first-level rings (delayed / direct trace), index n & 31
    float rB[32], rA[32];      // second-level rings, index n & 31
    float accF[NF], accS[8];
    float bF0, bF1, bS0, bS1;
    float curB[16], curA[16];  // samples n .. n+15 in flight (slot n & 15)
};

struct PairGeo {
    const float *inA, *inB;    // level-k samples [n][npix]
    float *outA, *outB;        // level-(k+2) samples [n][npix] or nullptr
    int k, nk, nk1, nk2;       // level and sample counts of levels k, k+1, k+2
    int sk0, sk1;              // direct samples [sk0, sk1) of level k
    int LF, LS;                // block lengths (samples) of levels k and k+1
    int lagF, lagS;            // first lag index of the two levels
};

__device__ __forceinline__ float c2_load(const float *in, int n, int nk, int npix, int pix)
{
    return n < nk ? __ldg(&in[(size_t)n * npix + pix]) : 0.f;
}

// Sample source of a pair kernel: level-k samples of the direct (a) and
// delayed (b) traces from the materialised FP32 streams.  prep(g) precedes
// the reads of group g's 16 samples (in order, jj = 0..15); acquire/release
// bracket the groups (hooks for a source that stages its data).
struct GlobalSrc {
    const float *inA, *inB;
    int nk, npix, pix;
    __device__ __forceinline__ void prep(int) {}
    __device__ __forceinline__ float a(int n, int) { return c2_load(inA, n, nk, npix, pix); }
    __device__ __forceinline__ float b(int n, int) { return c2_load(inB, n, nk, npix, pix); }
    __device__ __forceinline__ bool acquire(int) { return true; }
    __device__ __forceinline__ void release(int) {}
};

template <bool CCF, bool FIRST17, bool TWO, int QP, class Src>
__device__ __forceinline__ void c2_pair_group(const C2Ctx &c, const PairGeo &p, float *heads, int nt,
                                              PairReg<FIRST17> &R, int g, Src &src)
{
    constexpr int NF = PairReg<FIRST17>::NF, DF = PairReg<FIRST17>::DF;
    constexpr int PH0 = 16 * (QP & 1);
    constexpr int PH1 = 8 * QP;
    const int n0 = 16 * g;
    const bool dirF = (n0 - 16 >= p.sk0) && (n0 - 16 < p.sk1);          // direct samples n0-16 .. n0-1
    const bool dirS = TWO && (n0 - 32 >= p.sk0) && (n0 - 32 < p.sk1);   // second-level 8g-16 .. 8g-9
    src.prep(g + 1);
#pragma unroll
    for (int jj = 0; jj < 16; jj++) {
        const int n = n0 + jj;
        const float vB = R.curB[jj];
        R.wB[(PH0 + jj) & 31] = vB;
        if (CCF) {
            R.wA[(PH0 + jj) & 31] = R.curA[jj];
            R.curA[jj] = src.a(n + 16, jj);
        }
        R.curB[jj] = src.b(n + 16, jj);
        if (dirF) {
            // direct sample y = n - 16 with delayed samples y + DF .. y + 16 = n
            const float x0 = CCF ? R.wA[(PH0 + 16 + jj) & 31] : R.wB[(PH0 + 16 + jj) & 31];
#pragma unroll
            for (int d = 0; d < NF; d++) R.accF[d] = fmaf(x0, R.wB[(PH0 + 16 + jj + DF + d) & 31], R.accF[d]);
            R.bF0 += x0;
            R.bF1 += R.wB[(PH0 + 16 + jj) & 31];
        }
        if (TWO && (jj & 1)) {
            // second-level sample m = 8g + jj/2 from first-level samples n-1, n
            const int i1 = jj >> 1;
            const int m = 8 * g + i1;
            const bool ok = m < p.nk1;
            const float sB = ok ? R.wB[(PH0 + jj - 1) & 31] + R.wB[(PH0 + jj) & 31] : 0.f;
            R.rB[(PH1 + i1) & 31] = sB;
            if (CCF) R.rA[(PH1 + i1) & 31] = ok ? R.wA[(PH0 + jj - 1) & 31] + R.wA[(PH0 + jj) & 31] : 0.f;
            if (dirS) {
                // direct sample y1 = m - 16, delayed samples y1 + 9 .. y1 + 16 = m
                const float x1 = CCF ? R.rA[(PH1 + i1 + 16) & 31] : R.rB[(PH1 + i1 + 16) & 31];
#pragma unroll
                for (int l = 0; l < 8; l++) R.accS[l] = fmaf(x1, R.rB[(PH1 + i1 + 16 + 9 + l) & 31], R.accS[l]);
                R.bS0 += x1;
                R.bS1 += R.rB[(PH1 + i1 + 16) & 31];
            }
        }
    }
    // level-(k+2) samples 4g .. 4g+3 from second-level samples 8g .. 8g+7
    if (TWO && p.outB && c.valid) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int m2 = 4 * g + i;
            if (m2 >= (p.sk0 >> 2) && m2 < (p.sk1 >> 2) && m2 < p.nk2) {
                p.outB[(size_t)m2 * c.npix + c.pix] = R.rB[(PH1 + 2 * i) & 31] + R.rB[(PH1 + 2 * i + 1) & 31];
                if (CCF)
                    p.outA[(size_t)m2 * c.npix + c.pix] = R.rA[(PH1 + 2 * i) & 31] + R.rA[(PH1 + 2 * i + 1) & 31];
            }
        }
    }
    // heads of the segment's first blocks (its first 16 samples of either
    // level sit at ring positions 0..15)
    if (QP == 1 && n0 == p.sk0 + 16) {
        float h = 0.f;
        heads[0] = 0.f;
#pragma unroll
        for (int d = 1; d <= kP; d++) { h += R.wB[(d - 1) & 31]; heads[d * nt] = h; }
    }
    if (TWO && QP == 2 && n0 == p.sk0 + 32) {
        float h = 0.f;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            h += R.rB[i & 31];
            if (i + 1 >= 9) heads[(kP + 1 + i + 1 - 9) * nt] = h;
        }
    }
    // first-level block end: last direct sample y = n0 - 1; heads of the next
    // block are samples n0 .. n0 + d - 1 (this group)
    if (dirF && (n0 & (p.LF - 1)) == 0) {
        const int z = n0 / p.LF - 1;
#pragma unroll 1
        for (int l = 0; l < NF; l++) {
            const int d = DF + l;
            float nh = 0.f;
#pragma unroll
            for (int i = 0; i < kP; i++)
                if (i < d) nh += R.wB[(PH0 + i) & 31];
            float A = 0.f;
#pragma unroll
            for (int ll = 0; ll < NF; ll++)
                if (ll == l) A = R.accF[ll];
            float *hd = heads + d * nt;
            c2_block_stat(c, p.lagF + l, A, R.bF0, R.bF1 - hd[0] + nh, p.LF, z);
            hd[0] = nh;
        }
#pragma unroll
        for (int l = 0; l < NF; l++) R.accF[l] = 0.f;
        R.bF0 = 0.f;
        R.bF1 = 0.f;
    }
    // second-level block end: last direct sample y1 = 8g - 9; heads of the
    // next block are second-level samples 8g - 8 .. 8g - 9 + d
    if (dirS && ((8 * g - 8) & (p.LS - 1)) == 0) {
        const int z = (8 * g - 8) / p.LS - 1;
#pragma unroll 1
        for (int l = 0; l < 8; l++) {
            const int d = 9 + l;
            float nh = 0.f;
#pragma unroll
            for (int i = 1; i <= kP; i++)
                if (i <= d) nh += R.rB[(PH1 - 9 + i + 32) & 31];
            float A = 0.f;
#pragma unroll
            for (int ll = 0; ll < 8; ll++)
                if (ll == l) A = R.accS[ll];
            float *hd = heads + (kP + 1 + l) * nt;
            c2_block_stat(c, p.lagS + l, A, R.bS0, R.bS1 - hd[0] + nh, p.LS, z);
            hd[0] = nh;
        }
#pragma unroll
        for (int l = 0; l < 8; l++) R.accS[l] = 0.f;
        R.bS0 = 0.f;
        R.bS1 = 0.f;
    }
}

// First lag of levels (k, k+1) handled by one pair pass.
__host__ __device__ __forceinline__ int pair_lag0(int k, bool first17) { return first17 ? 0 : (kP + 1) + (k - 1) * 8; }

// One (pixel, segment) of levels k and k+1: the register-ring pass over the
// segment's level-k samples from `src`.  heads: this thread's heads (stride
// nt floats); sst / smon (optional): shared-memory block statistics (written
// back by the caller) and monitors of the pass's lags, from pair_lag0 on,
// stride nt.
template <bool CCF, bool FIRST17, bool TWO, class Src>
__device__ __forceinline__ void c2_pair_body(const C2Args &a, Src &src, float *outA, float *outB, int k, int pix,
                                             int seg, float *heads, int nt, float *sst = nullptr,
                                             const float2 *smon = nullptr)
{
    C2Ctx c;
    c2_ctx(c, a, pix, seg, k);
    if (sst) { c.sst = sst; c.sst_stride = nt; c.lag0 = pair_lag0(k, FIRST17); }
    if (smon) { c.smon = smon; c.smon_stride = nt; c.lag0 = pair_lag0(k, FIRST17); }
    PairGeo p;
    p.outA = outA;
    p.outB = outB;
    p.k = k;
    p.nk = a.numbin[k];
    p.nk1 = TWO ? a.numbin[k + 1] : 0;
    p.nk2 = (TWO && k + 2 < a.q) ? a.numbin[k + 2] : 0;
    const int s0 = seg << a.seg_log[k];
    const int s1 = s0 + (1 << a.seg_log[k]);
    p.sk0 = s0 >> k;
    p.sk1 = s1 >= a.num ? p.nk : (s1 >> k);
    p.LF = 1 << (c.ind - k);
    p.LS = 1 << (c.ind - k - 1);
    p.lagF = FIRST17 ? 0 : (kP + 1) + (k - 1) * 8;
    p.lagS = (kP + 1) + k * 8;

    if (c.valid) {
        for (int lag = p.lagF; lag < p.lagF + PairReg<FIRST17>::NF; lag++)
            for (int st = 0; st < kStatN; st++) c.stat(lag, st) = 0.f;
        if (TWO)
            for (int lag = p.lagS; lag < p.lagS + 8; lag++)
                for (int st = 0; st < kStatN; st++) c.stat(lag, st) = 0.f;
    }
    for (int f = 0; f < kHeadFields; f++) heads[f * nt] = 0.f;

    PairReg<FIRST17> R;
#pragma unroll
    for (int i = 0; i < 32; i++) { R.wB[i] = 0.f; R.wA[i] = 0.f; R.rB[i] = 0.f; R.rA[i] = 0.f; }
#pragma unroll
    for (int d = 0; d < PairReg<FIRST17>::NF; d++) R.accF[d] = 0.f;
#pragma unroll
    for (int l = 0; l < 8; l++) R.accS[l] = 0.f;
    R.bF0 = R.bF1 = R.bS0 = R.bS1 = 0.f;
    if (!src.acquire(0)) return;
    src.prep(p.sk0 / 16);
#pragma unroll
    for (int i = 0; i < 16; i++) {
        R.curA[i] = CCF ? src.a(p.sk0 + i, i) : 0.f;
        R.curB[i] = src.b(p.sk0 + i, i);
    }
    // groups of 16 samples: the segment's, then 48 more (the second level's
    // last direct samples need 16 second-level samples past the segment);
    // group r (relative) reads the samples of group r + 1
    const int g0 = p.sk0 / 16;
    int ng = (p.sk1 - p.sk0 + 48 + 15) / 16;
    ng = (ng + 3) & ~3;
    for (int r = 0; r < ng; r += 4) {
        const int g = g0 + r;
        if (!src.acquire(r + 1)) return;
        c2_pair_group<CCF, FIRST17, TWO, 0>(c, p, heads, nt, R, g, src);
        src.release(r);
        if (!src.acquire(r + 2)) return;
        c2_pair_group<CCF, FIRST17, TWO, 1>(c, p, heads, nt, R, g + 1, src);
        src.release(r + 1);
        if (!src.acquire(r + 3)) return;
        c2_pair_group<CCF, FIRST17, TWO, 2>(c, p, heads, nt, R, g + 2, src);
        src.release(r + 2);
        if (!src.acquire(r + 4)) return;
        c2_pair_group<CCF, FIRST17, TWO, 3>(c, p, heads, nt, R, g + 3, src);
        src.release(r + 3);
    }
    // the partial blocks at the end into the totals
#pragma unroll
    for (int l = 0; l < PairReg<FIRST17>::NF; l++) c2_add_total(c, p.lagF + l, R.accF[l]);
    if (TWO)
#pragma unroll
        for (int l = 0; l < 8; l++) c2_add_total(c, p.lagS + l, R.accS[l]);
}

template <bool CCF, bool FIRST17, bool TWO, int NT>
__global__ void __launch_bounds__(NT) c2_pair_kernel(C2Args a, const float *inA, const float *inB,
                                                     float *outA, float *outB, int k)
{
    constexpr int NL = (FIRST17 ? kP + 1 : 8) + (TWO ? 8 : 0);
    __shared__ float heads_sm[kHeadFields * NT];
    // block statistics and monitors of this pass's lags in shared memory: the
    // read-modify-writes at block ends stay on chip; written back at the end
    __shared__ float sst[NL * kStatN * NT];
    __shared__ float2 smon[NL * NT];
    const int nt = blockDim.x, tid = threadIdx.x;
    const int pix = blockIdx.x * nt + tid, seg = blockIdx.y;
    if (pix >= a.npix) return;          // no block-wide synchronisation below
    if ((seg << a.seg_log[k]) >= a.num) return;
    const int lag0 = pair_lag0(k, FIRST17);
    {
        const float4 *m = a.mon + (size_t)pix * a.chanum + lag0;
        for (int l = 0; l < NL; l++) {
            const float4 v = __ldg(&m[l]);
            smon[l * nt + tid] = make_float2(v.x, v.y);
        }
    }
    GlobalSrc src{CCF ? inA : inB, inB, a.numbin[k], a.npix, pix};
    c2_pair_body<CCF, FIRST17, TWO>(a, src, outA, outB, k, pix, seg, heads_sm + tid, nt, sst + tid, smon + tid);
    float *gst = a.o.stats + (size_t)seg * a.stat_stride;
    for (int l = 0; l < NL; l++)
        for (int st = 0; st < kStatN; st++)
            stat_ref(gst, a.npix, lag0 + l, st, pix) = sst[(size_t)(l * kStatN + st) * nt + tid];
}

// ---------------------------------------------------------------------------
// Tail kernel: one level k >= k0 of one (pixel, segment) per thread, for the
// top levels whose blocks may be as short as one sample.  The thread builds
// its level-k samples from the level-k0 stream (sums of 2^(k-k0) samples),
// keeps a ring of its last 32 samples in shared memory and its lags' block
// sums and block statistics in registers; the statistics are written once.
// ---------------------------------------------------------------------------
// (8 warps per SM at least: 128 registers, a few spilled, against 160 at
// 6 warps -- the kernel waits on its loads, 6.44 -> 6.18 ms for the chain)
template <bool CCF, int NT>
__global__ void __launch_bounds__(NT, 512 / NT) c2_tail_kernel(C2Args a, const float *inA, const float *inB, int k0)
{
    __shared__ float ring_sm[(CCF ? 2 : 1) * 32 * NT];
    const int tid = threadIdx.x;
    const int pix = blockIdx.x * NT + tid, seg = blockIdx.y, k = k0 + blockIdx.z;
    if (pix >= a.npix || k >= a.q) return;          // no block-wide synchronisation below
    float *rb = ring_sm + tid;
    float *ra = CCF ? ring_sm + 32 * NT + tid : rb;
    if (!CCF) inA = inB;
    C2Ctx c;
    c2_ctx(c, a, pix, seg, k);
    const int s0 = seg << a.seg_log[k];
    if (s0 >= a.num) return;
    const int s1 = min(s0 + (1 << a.seg_log[k]), a.num);
    const int nkk = a.numbin[k], nk0 = a.numbin[k0];
    const int ys0 = s0 >> k, ys1 = (s1 >= a.num) ? nkk : (s1 >> k);
    const int m = 1 << (k - k0);
    const int lag0 = (kP + 1) + (k - 1) * 8;
    const int lk = c.ind - k;
    const int L = lk > 0 ? (1 << lk) : 1;

    float ma[8], mb[8];
#pragma unroll
    for (int l = 0; l < 8; l++) {
        const float4 mm = __ldg(&c.mon[lag0 + l]);
        ma[l] = mm.x;
        mb[l] = mm.y;
    }
    float acc[8], head[8], thi[8], tlo[8], S1[8], S2[8], rr[8];
#pragma unroll
    for (int l = 0; l < 8; l++) {
        acc[l] = head[l] = thi[l] = tlo[l] = S1[l] = S2[l] = rr[l] = 0.f;
    }
    float b0 = 0.f, b1 = 0.f;

    // samples ys0 .. ys1 + 15 (the last direct samples' delayed partners);
    // samples from nkk on are zero.  Loads are issued 8 samples at a time.
    const int nend = ys1 + 16;
#pragma unroll 1
    for (int nb = ys0; nb < nend; nb += 8) {
        float vb[8], va[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            vb[u] = 0.f;
            va[u] = 0.f;
            const int n = nb + u;
            if (n < nkk && n < nend) {
                if (m <= 8) {
                    // pairwise sums, as the levels are built (java:9467-9476)
                    float wb[8], wa[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const int q = n * m + i;
                        const bool in = i < m && q < nk0;
                        wb[i] = in ? __ldg(&inB[(size_t)q * a.npix + pix]) : 0.f;
                        wa[i] = (CCF && in) ? __ldg(&inA[(size_t)q * a.npix + pix]) : 0.f;
                    }
#pragma unroll
                    for (int w = 1; w < 8; w *= 2)
#pragma unroll
                        for (int i = 0; i < 8; i += 2 * w) {
                            wb[i] += wb[i + w];
                            wa[i] += wa[i + w];
                        }
                    vb[u] = wb[0];
                    va[u] = wa[0];
                } else {
                    for (int i = 0; i < m; i++) {
                        const int q = n * m + i;
                        if (q < nk0) {
                            vb[u] += __ldg(&inB[(size_t)q * a.npix + pix]);
                            if (CCF) va[u] += __ldg(&inA[(size_t)q * a.npix + pix]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int n = nb + u;
            if (n >= nend) break;
            rb[(n & 31) * NT] = vb[u];
            if (CCF) ra[(n & 31) * NT] = va[u];
            const int y = n - 16;
            if (y < ys0) continue;
            if (y == ys0) {
                float h = 0.f;
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    h += rb[((y + i) & 31) * NT];
                    if (i + 1 >= 9) head[i + 1 - 9] = h;
                }
            }
            const float x0 = ra[(y & 31) * NT];
#pragma unroll
            for (int l = 0; l < 8; l++) acc[l] = fmaf(x0, rb[((y + 9 + l) & 31) * NT], acc[l]);
            b0 += x0;
            b1 += rb[(y & 31) * NT];
            if (((y + 1) & (L - 1)) == 0) {
                // heads of the next block: sums of the delayed samples y+1 .. y+d
                float nh[8], h = 0.f;
#pragma unroll
                for (int i = 1; i <= 16; i++) {
                    h += rb[((y + i) & 31) * NT];
                    if (i >= 9) nh[i - 9] = h;
                }
                const int z = y / L;
                const bool stat = z < c.pnum;
#pragma unroll
                for (int l = 0; l < 8; l++) {
                    const float D = b1 - head[l] + nh[l];
                    const float P = (acc[l] - mb[l] * b0 - ma[l] * D + (float)L * ma[l] * mb[l]) / (float)L;
                    ff t = {thi[l], tlo[l]};
                    ff_add(t, acc[l]);
                    thi[l] = t.hi;
                    tlo[l] = t.lo;
                    if (stat) {
                        if (z == c.zfirst) rr[l] = P;
                        const float dv = P - rr[l];
                        S1[l] += dv;
                        S2[l] = fmaf(dv, dv, S2[l]);
                        if (c.gls)
                            c.bprod[((size_t)pix * (c.chanum - 1) + (lag0 + l - 1)) * c.pnum_stride + z] = P;
                    }
                    head[l] = nh[l];
                    acc[l] = 0.f;
                }
                b0 = 0.f;
                b1 = 0.f;
            }
        }
    }
#pragma unroll
    for (int l = 0; l < 8; l++) {
        ff t = {thi[l], tlo[l]};
        ff_add(t, acc[l]);
        stat_ref(c.stats, c.npix, lag0 + l, 0, pix) = t.hi;
        stat_ref(c.stats, c.npix, lag0 + l, 1, pix) = t.lo;
        stat_ref(c.stats, c.npix, lag0 + l, 2, pix) = S1[l];
        stat_ref(c.stats, c.npix, lag0 + l, 3, pix) = S2[l];
        stat_ref(c.stats, c.npix, lag0 + l, 4, pix) = rr[l];
    }
}

// ---------------------------------------------------------------------------
// Generic-P level kernel (the plugin's P = 32, java:1022-1024): one (pixel,
// level k, group of up to 8 delays) per thread over the whole frame range
// (one segment).  Level 0 has delays 0..P, level k >= 1 delays P/2+1..P
// (java:7391-7424).  The thread builds its level-k samples from the level-0
// stream (sums of 2^k samples, pairwise within groups of 8), keeps a ring of
// its last 2P samples in shared memory and its delays' block sums and block
// statistics in registers, like the tail kernel.
// ---------------------------------------------------------------------------
template <bool CCF, int P>
__global__ void __launch_bounds__(64) cg_kernel(C2Args a, const float *inA, const float *inB)
{
    constexpr int NT = 64;
    constexpr int RS = 2 * P;                       // ring (power of two, > the largest delay)
    constexpr int G0 = (P + 1 + 7) / 8;             // level-0 groups: delays 0..P
    constexpr int GK = P / 2 / 8;                   // groups of an upper level
    __shared__ float ring_sm[(CCF ? 2 : 1) * RS * NT];
    const int tid = threadIdx.x;
    const int pix = blockIdx.x * NT + tid;
    const int gy = blockIdx.y;
    int k, dlo, nd;
    if (gy < G0) { k = 0; dlo = 8 * gy; nd = min(8, P + 1 - dlo); }
    else { k = 1 + (gy - G0) / GK; dlo = P / 2 + 1 + 8 * ((gy - G0) % GK); nd = 8; }
    if (pix >= a.npix || k >= a.q) return;          // no block-wide synchronisation below
    float *rb = ring_sm + tid;
    float *ra = CCF ? ring_sm + RS * NT + tid : rb;
    if (!CCF) inA = inB;
    C2Ctx c;
    c2_ctx(c, a, pix, 0, k);
    const int nkk = a.numbin[k], nk0 = a.numbin[0];
    const int m = 1 << k;
    const int lag0 = k == 0 ? dlo : (P + 1) + (k - 1) * (P / 2) + (dlo - (P / 2 + 1));
    const int dmax = dlo + nd - 1;
    const int lk = c.ind - k;
    const int L = lk > 0 ? (1 << lk) : 1;

    float ma[8], mb[8];
#pragma unroll
    for (int l = 0; l < 8; l++) {
        const float4 mm = __ldg(&c.mon[lag0 + min(l, nd - 1)]);
        ma[l] = mm.x;
        mb[l] = mm.y;
    }
    float acc[8], head[8], thi[8], tlo[8], S1[8], S2[8], rr[8];
#pragma unroll
    for (int l = 0; l < 8; l++) acc[l] = head[l] = thi[l] = tlo[l] = S1[l] = S2[l] = rr[l] = 0.f;
    float b0 = 0.f, b1 = 0.f;

    // samples 0 .. nkk - 1 + dmax (samples from nkk on are zero)
    const int nend = nkk + dmax;
#pragma unroll 1
    for (int n = 0; n < nend; n++) {
        float vb = 0.f, va = 0.f;
        if (n < nkk) {
            for (int q0 = n * m; q0 < n * m + m; q0 += 8) {
                float wb[8], wa[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int q = q0 + i;
                    const bool in = i < m && q < nk0;
                    wb[i] = in ? __ldg(&inB[(size_t)q * a.npix + pix]) : 0.f;
                    wa[i] = (CCF && in) ? __ldg(&inA[(size_t)q * a.npix + pix]) : 0.f;
                }
#pragma unroll
                for (int w = 1; w < 8; w *= 2)
#pragma unroll
                    for (int i = 0; i < 8; i += 2 * w) {
                        wb[i] += wb[i + w];
                        wa[i] += wa[i + w];
                    }
                vb += wb[0];
                va += wa[0];
            }
        }
        rb[(n & (RS - 1)) * NT] = vb;
        if (CCF) ra[(n & (RS - 1)) * NT] = va;
        const int y = n - dmax;
        if (y < 0) continue;
        if (y == 0) {
            // heads of the first block: sums of the delayed samples 0 .. d-1
            float h = 0.f;
#pragma unroll
            for (int l = 0; l < 8; l++) head[l] = 0.f;
            for (int i = 0; i < dmax; i++) {
                h += rb[(i & (RS - 1)) * NT];
#pragma unroll
                for (int l = 0; l < 8; l++)
                    if (dlo + l == i + 1) head[l] = h;
            }
        }
        const float x0 = ra[(y & (RS - 1)) * NT];
#pragma unroll
        for (int l = 0; l < 8; l++) acc[l] = fmaf(x0, rb[((y + dlo + l) & (RS - 1)) * NT], acc[l]);
        b0 += x0;
        b1 += rb[(y & (RS - 1)) * NT];
        if (((y + 1) & (L - 1)) == 0) {
            // heads of the next block: sums of the delayed samples y+1 .. y+d
            float nh[8], h = 0.f;
#pragma unroll
            for (int l = 0; l < 8; l++) nh[l] = 0.f;
            for (int i = 1; i <= dmax; i++) {
                h += rb[((y + i) & (RS - 1)) * NT];
#pragma unroll
                for (int l = 0; l < 8; l++)
                    if (dlo + l == i) nh[l] = h;
            }
            const int z = y / L;
            const bool stat = z < c.pnum;
#pragma unroll
            for (int l = 0; l < 8; l++) {
                const float D = b1 - head[l] + nh[l];
                const float Pz = (acc[l] - mb[l] * b0 - ma[l] * D + (float)L * ma[l] * mb[l]) / (float)L;
                ff t = {thi[l], tlo[l]};
                ff_add(t, acc[l]);
                thi[l] = t.hi;
                tlo[l] = t.lo;
                if (stat && l < nd) {
                    if (z == 0) rr[l] = Pz;
                    const float dv = Pz - rr[l];
                    S1[l] += dv;
                    S2[l] = fmaf(dv, dv, S2[l]);
                    if (c.gls && lag0 + l >= 1)
                        c.bprod[((size_t)pix * (c.chanum - 1) + (lag0 + l - 1)) * c.pnum_stride + z] = Pz;
                }
                head[l] = nh[l];
                acc[l] = 0.f;
            }
            b0 = 0.f;
            b1 = 0.f;
        }
    }
#pragma unroll
    for (int l = 0; l < 8; l++) {
        if (l >= nd) break;
        ff t = {thi[l], tlo[l]};
        ff_add(t, acc[l]);
        stat_ref(c.stats, c.npix, lag0 + l, 0, pix) = t.hi;
        stat_ref(c.stats, c.npix, lag0 + l, 1, pix) = t.lo;
        stat_ref(c.stats, c.npix, lag0 + l, 2, pix) = S1[l];
        stat_ref(c.stats, c.npix, lag0 + l, 3, pix) = S2[l];
        stat_ref(c.stats, c.npix, lag0 + l, 4, pix) = rr[l];
    }
}

// ---------------------------------------------------------------------------
// Finalise: segments combined per (pixel, lag): product totals, block
// statistics brought to one shift (FP64), outputs as calculateCF
// (java:9491-9531).
// ---------------------------------------------------------------------------
__global__ void c2_finalize_kernel(C2Args a)
{
    // lag-major threads: the segment statistics [lag][stat][pixel] are read
    // coalesced (they are most of this kernel's traffic)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.npix * a.chanum) return;
    const int lag = i / a.npix, pix = i % a.npix;
    const int ind = a.blk_ind[pix];
    const int pnum = a.li->pnum_by_ind[ind];
    const int level = lag <= a.p ? 0 : 1 + (lag - (a.p + 1)) / (a.p / 2);
    const int sl = a.seg_log[level];
    const int nseg = (a.num + (1 << sl) - 1) >> sl;
    double A = 0.0, S1 = 0.0, S2 = 0.0, r = 0.0;
    bool have_r = false;
    for (int sg = 0; sg < nseg; sg++) {
        float *st = a.o.stats + sg * a.stat_stride;
        A += (double)stat_ref(st, a.npix, lag, 0, pix) + (double)stat_ref(st, a.npix, lag, 1, pix);
        const int s0 = sg << sl, s1 = min(s0 + (1 << sl), a.num);
        const int z0 = s0 >> ind, z1 = (s1 + (1 << ind) - 1) >> ind;
        const int cnt = max(0, min(pnum, z1) - z0);
        if (cnt == 0) continue;
        const double rs = stat_ref(st, a.npix, lag, 4, pix);
        const double s1s = stat_ref(st, a.npix, lag, 2, pix), s2s = stat_ref(st, a.npix, lag, 3, pix);
        if (!have_r) { r = rs; have_r = true; }
        const double dr = rs - r;
        S1 += s1s + cnt * dr;
        S2 += s2s + 2.0 * dr * s1s + cnt * dr * dr;
    }
    const float4 m = a.mon[(size_t)pix * a.chanum + lag];
    const double n = a.li->prodnum[lag];
    const double dmDm = (double)m.z * (double)m.w;
    const double sumprod = A - n * (double)m.x * (double)m.y;
    const double corav = sumprod / (n * dmDm);
    const double pn = pnum;
    const double bv = (S2 / pn - (S1 / pn) * (S1 / pn)) / ((pn - 1) * dmDm * dmDm);
    double acf = corav;
    if (a.o.gls) acf = (lag == 0) ? 0.0 : (S1 + pn * r) / (pn * dmDm);   // mcov (java:9526-9531)
    if (a.o.acf) a.o.acf[(size_t)pix * a.chanum + lag] = acf;
    if (a.o.var) a.o.var[(size_t)pix * a.chanum + lag] = bv;
    if (a.o.sd) a.o.sd[(size_t)pix * a.chanum + lag] = sqrt(bv);
    if (lag == 1) {
        if (a.o.nb_mean) a.o.nb_mean[pix] = m.z;
        if (a.o.nb_cov) a.o.nb_cov[pix] = sumprod / n;
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
// The chain needs blocks of at least 16 level-0 and 8 level-1 samples
// (ind >= Q-1 >= 4).
bool corr2_supported(const Job &j) { return j.p == kP && j.q >= 5; }
// P = 32: the generic level kernel (any Q)
bool corrg_supported(const Job &j) { return j.p == 32; }

namespace {
struct Plan2 {
    int npair;                // pair kernels (levels 0-1, then 2-3 when Q >= 7)
    int k_tail;               // first level of the tail kernel (Q: none)
    int seg_log[kMaxLevels];
    int nseg_max;
};

Plan2 plan2(const Job &j)
{
    Plan2 p;
    // every pixel's block length divides 2^base0 frames; the tile multiplies
    // the pair kernels' segments by 2^c2_seg_extra and the tail kernel's by
    // 2^c2_tail_extra
    const int base0 = max(j.blocknum - 1, j.q - 1);
    const int base = base0 + min(max(j.c2_seg_extra, 0), kMaxSegExtra);
    const int base_tail = base0 + min(max(j.c2_tail_extra, 0), kMaxSegExtra);
    p.npair = (j.q >= 7) ? 2 : 1;
    p.k_tail = 2 * p.npair;
    for (int k = 0; k < kMaxLevels; k++) p.seg_log[k] = 0;
    for (int i = 0; i < p.npair; i++) {
        const int k = 2 * i;
        const int sl = max(base, k + 6);            // segments start at multiples of 64 level-k samples
        p.seg_log[k] = p.seg_log[k + 1] = sl;
    }
    if (p.k_tail < j.q) {
        const int sl = max(base_tail, p.k_tail);
        for (int k = p.k_tail; k < j.q; k++) p.seg_log[k] = sl;
    }
    p.nseg_max = 1;
    for (int k = 0; k < j.q; k++)
        p.nseg_max = max(p.nseg_max, (j.num + (1 << p.seg_log[k]) - 1) >> p.seg_log[k]);
    return p;
}
}  // namespace

int corr2_nseg(const Job &j) { return plan2(j).nseg_max; }

int corr_kernel_count(const Job &j)
{
    if (corrg_supported(j)) return 2;
    if (!corr2_supported(j)) return 1;
    const Plan2 p = plan2(j);
    return p.npair + (p.k_tail < j.q ? 1 : 0) + 1;   // pair kernels, tail, finalise
}

size_t corr_stats_floats(const Job &j)
{
    const size_t one = (size_t)j.chanum * kStatN * j.npix;
    return corr2_supported(j) ? one * corr2_nseg(j) : one;
}

// Binned sample streams, per trace: s2 (num/4 x npix) and s4 (num/16 x
// npix), written by the pair kernels for the next level pair.
size_t corr_stream_floats(const Job &j)
{
    if (!corr2_supported(j)) return 1;
    const size_t tr = j.is_ccf ? 2 : 1;
    return tr * (size_t)j.npix * ((size_t)(j.num >> 2) + (size_t)(j.num >> 4) + 3);
}

// The corrected level-0 stream s0[trace][frame][pixel] (imfcs_stream.cu).
size_t level0_stream_floats(const Job &j) { return (size_t)(j.is_ccf ? 2 : 1) * j.npix * j.num; }

// One pair kernel of the chain: variant 0 = levels 0-1, 1 = two upper
// levels, 2 = one upper level (the last).
template <int NT>
static void launch_pair(bool ccf, int variant, dim3 grid, cudaStream_t stream, const C2Args &a, const float *ia,
                        const float *ib, float *oa, float *ob, int k)
{
    if (ccf) {
        if (variant == 0) c2_pair_kernel<true, true, true, NT><<<grid, NT, 0, stream>>>(a, ia, ib, oa, ob, k);
        else if (variant == 1) c2_pair_kernel<true, false, true, NT><<<grid, NT, 0, stream>>>(a, ia, ib, oa, ob, k);
        else c2_pair_kernel<true, false, false, NT><<<grid, NT, 0, stream>>>(a, ia, ib, oa, ob, k);
    } else {
        if (variant == 0) c2_pair_kernel<false, true, true, NT><<<grid, NT, 0, stream>>>(a, ia, ib, oa, ob, k);
        else if (variant == 1) c2_pair_kernel<false, false, true, NT><<<grid, NT, 0, stream>>>(a, ia, ib, oa, ob, k);
        else c2_pair_kernel<false, false, false, NT><<<grid, NT, 0, stream>>>(a, ia, ib, oa, ob, k);
    }
}

// The generic-P correlator: level kernel over the whole frame range, then
// the finalise kernel (one segment).

cudaError_t launch_corrg(const Job &j, const LagInfo *li, const float *s0, const float4 *mon, const int *blk_ind,
                         const CorrOut &o, cudaStream_t stream)
{
    C2Args a;
    memset(&a, 0, sizeof(a));
    a.o = o;
    a.mon = mon;
    a.blk_ind = blk_ind;
    a.li = li;
    a.npix = j.npix;
    a.chanum = j.chanum;
    a.p = j.p;
    a.q = j.q;
    a.num = j.num;
    {
        int nb = j.num;
        for (int k = 0; k < j.q; k++) { a.numbin[k] = nb; nb /= 2; }
    }
    for (int k = 0; k < kMaxLevels; k++) a.seg_log[k] = 30;   // one segment
    a.stat_stride = (size_t)j.chanum * kStatN * j.npix;
    const float *s0a = s0, *s0b = j.is_ccf ? s0 + (size_t)j.npix * j.num : s0;
    constexpr int P = 32;
    const dim3 grid((j.npix + 63) / 64, (P + 1 + 7) / 8 + (j.q - 1) * (P / 16));
    if (j.is_ccf) cg_kernel<true, P><<<grid, 64, 0, stream>>>(a, s0a, s0b);
    else cg_kernel<false, P><<<grid, 64, 0, stream>>>(a, s0a, s0b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int n = j.npix * j.chanum;
    c2_finalize_kernel<<<(n + 255) / 256, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_corr2(const Job &j, const LagInfo *li, const float *s0, const float4 *mon, const int *blk_ind,
                         const CorrOut &o, float *streams, cudaStream_t stream)
{
    const Plan2 pl = plan2(j);
    C2Args a;
    memset(&a, 0, sizeof(a));
    a.o = o;
    a.mon = mon;
    a.blk_ind = blk_ind;
    a.li = li;
    a.npix = j.npix;
    a.chanum = j.chanum;
    a.p = j.p;
    a.q = j.q;
    a.num = j.num;
    {
        int nb = j.num;
        for (int k = 0; k < j.q; k++) { a.numbin[k] = nb; nb /= 2; }
    }
    for (int k = 0; k < kMaxLevels; k++) a.seg_log[k] = pl.seg_log[k];
    a.stat_stride = (size_t)j.chanum * kStatN * j.npix;

    const size_t tr = j.is_ccf ? 2 : 1;
    const size_t np = j.npix;
    const float *s0a = s0, *s0b = j.is_ccf ? s0 + np * j.num : s0;
    float *s2a = streams, *s2b = j.is_ccf ? s2a + np * (j.num >> 2) : s2a;
    float *s4a = s2a + tr * np * (j.num >> 2), *s4b = j.is_ccf ? s4a + np * (j.num >> 4) : s4a;
    cudaError_t e = cudaSuccess;

    const int nt = j.c2_cta == 32 ? 32 : kC2Threads;
    const int pgx = (j.npix + nt - 1) / nt;
    for (int i = 0; i < pl.npair; i++) {
        const int k = 2 * i;
        const float *ia = i ? s2a : s0a, *ib = i ? s2b : s0b;
        float *oa = (k + 2 < j.q) ? (i ? s4a : s2a) : nullptr;
        float *ob = (k + 2 < j.q) ? (i ? s4b : s2b) : nullptr;
        const dim3 grid(pgx, (j.num + (1 << pl.seg_log[k]) - 1) >> pl.seg_log[k]);
        const int variant = (i == 0) ? 0 : (k + 1 < j.q ? 1 : 2);
        if (nt == 32) launch_pair<32>(j.is_ccf, variant, grid, stream, a, ia, ib, oa, ob, k);
        else launch_pair<kC2Threads>(j.is_ccf, variant, grid, stream, a, ia, ib, oa, ob, k);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (pl.k_tail < j.q) {
        const int k0 = pl.k_tail;
        const float *ia = (k0 == 2) ? s2a : s4a, *ib = (k0 == 2) ? s2b : s4b;
        const dim3 grid(pgx, (j.num + (1 << pl.seg_log[k0]) - 1) >> pl.seg_log[k0], j.q - k0);
        if (nt == 32) {
            if (j.is_ccf) c2_tail_kernel<true, 32><<<grid, 32, 0, stream>>>(a, ia, ib, k0);
            else c2_tail_kernel<false, 32><<<grid, 32, 0, stream>>>(a, ia, ib, k0);
        } else {
            if (j.is_ccf) c2_tail_kernel<true, kC2Threads><<<grid, kC2Threads, 0, stream>>>(a, ia, ib, k0);
            else c2_tail_kernel<false, kC2Threads><<<grid, kC2Threads, 0, stream>>>(a, ia, ib, k0);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const int n = j.npix * j.chanum;
    c2_finalize_kernel<<<(n + 255) / 256, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace imfcs
