// imfcs_capi.cu -- C ABI of libimfcs_gb300.so: plans, the whole-path
// pipeline, and the entry points that replace the GpufitImFCS natives.
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "imfcs_args.h"
#include "imfcs_gb300.h"
#include "imfcs_host.h"

using namespace imfcs;

// ---------------------------------------------------------------------------
// Errors: per-thread message, like getLastError (agpufitjni.cu:4643).
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

namespace imfcs {
void set_error(const std::string &msg) { g_last_error = msg; }
std::string cuda_msg(cudaError_t e, const char *what)
{
    return std::string(what) + ": " + cudaGetErrorString(e);
}
}  // namespace imfcs

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) { set_error(cuda_msg(_e, #call)); return 1; } \
    } while (0)

extern "C" const char *imfcs_get_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// Lag tables (java:7340-7346, 7391-7424) and the derived structure.
// ---------------------------------------------------------------------------
namespace imfcs {

bool build_lag_info(int p, int q, int num, LagInfo &li, int &chanum, int &blocknum,
                    std::string &err)
{
    memset(&li, 0, sizeof(li));
    if (p != 16 && p != 32) { err = "correlator P must be 16 or 32"; return false; }
    if (q < 2 || q > 8) { err = "correlator Q must be in 2..8 in this build"; return false; }
    chanum = (int)(p + (q - 1) * (double)p / 2 + 1);
    if (chanum > kMaxChan) { err = "too many correlation channels"; return false; }
    // "Not enough frames" (java:7315)
    if ((num - pow(2, q - 1) * p / 2 - p / 4 * pow(2, q)) / pow(2, q - 1) < 1) {
        err = "Not enough frames";
        return false;
    }
    const int base = p, hbase = p / 2, lagnum = q;
    std::vector<int> lag(chanum);
    std::vector<double> samp(chanum), mtab(chanum);
    for (int x = 0; x <= hbase; x++) lag[x] = x;
    for (int x = 1; x <= lagnum; x++)
        for (int y = 1; y <= hbase; y++)
            lag[x * hbase + y] = (int)(pow(2, x - 1) * y + (base / 4) * pow(2, x));
    for (int x = 0; x <= base; x++) samp[x] = 1;
    for (int x = 2; x <= lagnum; x++)
        for (int y = 1; y <= hbase; y++) samp[x * hbase + y] = pow(2, x - 1);
    for (int x = 0; x < chanum; x++) mtab[x] = (int)floor((num - lag[x]) / samp[x]);
    li.nlevels = q;
    int nb = num;
    for (int k = 0; k < q; k++) {
        if (k > 0) nb = nb / 2;
        li.numbin[k] = nb;
    }
    std::vector<int> pos;
    for (int x = 0; x < chanum; x++) {
        int k = (int)lround(log2(samp[x]));
        li.lag[x] = lag[x];
        li.level[x] = k;
        li.del[x] = lag[x] / (int)samp[x];
        li.prodnum[x] = li.numbin[k] - li.del[x];
        pos.push_back(li.prodnum[x] << k);
        pos.push_back(lag[x]);
        pos.push_back(li.numbin[k] << k);
    }
    pos.push_back(num - 2);
    pos.push_back(num - 1);
    std::sort(pos.begin(), pos.end());
    pos.erase(std::unique(pos.begin(), pos.end()), pos.end());
    if ((int)pos.size() > kMaxSnap) { err = "too many snapshot positions"; return false; }
    for (size_t i = 0; i < pos.size(); i++) li.snap_pos[i] = pos[i];
    li.nsnap = (int)pos.size();
    auto idx = [&](int v) { return (int)(std::lower_bound(pos.begin(), pos.end(), v) - pos.begin()); };
    for (int x = 0; x < chanum; x++) {
        int k = li.level[x];
        li.snap_dir_end[x] = idx(li.prodnum[x] << k);
        li.snap_del_beg[x] = idx(lag[x]);
        li.snap_del_end[x] = idx(li.numbin[k] << k);
    }
    li.snap_tm2 = idx(num - 2);
    li.snap_tm1 = idx(num - 1);
    // pnum for every block index (java:9435)
    for (int ind = 0; ind < kMaxBlockLevels; ind++)
        li.pnum_by_ind[ind] = (int)floor(mtab[chanum - 1] /
                                         pow(2, fmax(ind - log(samp[chanum - 1]) / log(2), 0)));
    blocknum = (int)floor(log(mtab[1]) / log(2)) - 2;
    if (blocknum < 4) { err = "too few frames for the blocking transform"; return false; }
    if (blocknum > kMaxBlockLevels) { err = "too many blocking levels"; return false; }
    return true;
}

static void legendre_d(double u, int order, double *out)
{
    out[0] = 1.0;
    if (order >= 1) out[1] = u;
    for (int n = 1; n < order; n++) out[n + 1] = ((2 * n + 1) * u * out[n] - n * out[n - 1]) / (n + 1);
}

// Least-squares projection in the Legendre basis of u = t*uscale + uoff over
// the averaged-trace times t_x = frametime (x + 0.5) ave (java:9853), FP64:
// proj = (Phi^T Phi)^-1 Phi^T.
void legendre_projection(int order, int nopit, int ave, double frametime, double *proj,
                         double &uscale, double &uoff)
{
    const int k = order + 1;
    double t0 = frametime * 0.5 * ave, t1 = frametime * (nopit - 0.5) * ave;
    uscale = (t1 > t0) ? 2.0 / (t1 - t0) : 1.0;
    uoff = -1.0 - t0 * uscale;
    std::vector<double> phi((size_t)nopit * k), g(k * k, 0.0);
    for (int x = 0; x < nopit; x++) {
        double u = frametime * (x + 0.5) * ave * uscale + uoff;
        legendre_d(u, order, &phi[(size_t)x * k]);
    }
    for (int a = 0; a < k; a++)
        for (int b = 0; b < k; b++) {
            double s = 0.0;
            for (int x = 0; x < nopit; x++) s += phi[(size_t)x * k + a] * phi[(size_t)x * k + b];
            g[a * k + b] = s;
        }
    // invert g (SPD, well conditioned) by Gauss-Jordan
    std::vector<double> inv(k * k, 0.0);
    for (int i = 0; i < k; i++) inv[i * k + i] = 1.0;
    for (int c = 0; c < k; c++) {
        int pr = c;
        for (int r = c + 1; r < k; r++) if (fabs(g[r * k + c]) > fabs(g[pr * k + c])) pr = r;
        for (int q = 0; q < k; q++) { std::swap(g[c * k + q], g[pr * k + q]); std::swap(inv[c * k + q], inv[pr * k + q]); }
        double d = g[c * k + c];
        for (int q = 0; q < k; q++) { g[c * k + q] /= d; inv[c * k + q] /= d; }
        for (int r = 0; r < k; r++) {
            if (r == c) continue;
            double f = g[r * k + c];
            for (int q = 0; q < k; q++) { g[r * k + q] -= f * g[c * k + q]; inv[r * k + q] -= f * inv[c * k + q]; }
        }
    }
    for (int a = 0; a < k; a++)
        for (int x = 0; x < nopit; x++) {
            double s = 0.0;
            for (int b = 0; b < k; b++) s += inv[a * k + b] * phi[(size_t)x * k + b];
            proj[(size_t)a * nopit + x] = s;
        }
}

// Basis values at the correction times t = frametime (f + 1.5) of frames
// f = 0..num-1 (java:9747: x + 0.5 with 1-based x).
void legendre_basis_table(int order, int num, double frametime, double uscale, double uoff,
                          float *table)
{
    const int k = order + 1;
    double lb[kMaxPoly + 1];
    for (int f = 0; f < num; f++) {
        legendre_d(frametime * (f + 1.5) * uscale + uoff, order, lb);
        for (int i = 0; i < k; i++) table[(size_t)f * k + i] = (float)lb[i];
    }
}

}  // namespace imfcs

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------
static int device_sms()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

extern "C" int imfcs_chanum(int p, int q) { return (int)(p + (q - 1) * (double)p / 2 + 1); }

extern "C" int imfcs_is_cuda_available(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return 0;
    }
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) return 0;
    return (p.major * 10 + p.minor) >= 100 ? 1 : 0;
}

extern "C" int imfcs_get_cuda_version(int *runtime_version, int *driver_version)
{
    int rt = 0, dr = 0;
    CK(cudaRuntimeGetVersion(&rt));
    CK(cudaDriverGetVersion(&dr));
    if (runtime_version) *runtime_version = rt;
    if (driver_version) *driver_version = dr;
    return 0;
}

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
};

struct imfcs_plan {
    imfcs_config cfg;
    Job job;
    LagInfo li;
    LagInfo *li_dev = nullptr;
    int chanum = 0, npix = 0, nseg = 0, nbseg = 0, pnum_max = 0, nfitpts = 0, k = 0;
    int idx[IMFCS_NPARAM];
    int num_sms = 1;
    int launches = 0;                 // kernels launched by the last execute
    double uscale = 1, uoff = 0;
    bool given_bleach = false;
    std::vector<DevBuf> bufs;
    size_t bytes = 0;
    // scratch
    float *trace = nullptr, *bparams = nullptr, *basis = nullptr;
    double *proj = nullptr;
    int *snap_pos = nullptr;
    float2 *segtot = nullptr, *snap_part = nullptr;
    int *segbad = nullptr, *snap_bad = nullptr;   // non-finite frames per segment / snapshot partial
    float4 *mon = nullptr, *blkmon = nullptr;
    float *s1 = nullptr, *s2 = nullptr, *segsum = nullptr;
    int *blk_ind = nullptr, *blk_ok = nullptr;
    float *stats = nullptr, *bprod = nullptr, *streams = nullptr, *s0 = nullptr;
    float *linv = nullptr, *ytrans = nullptr;
    int *gls_ok = nullptr;
    float *fit_y = nullptr, *fit_w = nullptr, *fit_x = nullptr, *fit_x_gls = nullptr;
    float *fit_init = nullptr, *fit_par = nullptr, *fit_chi2 = nullptr, *fit_hess = nullptr;
    int *fit_state = nullptr, *fit_iter = nullptr;
    float *lagtime = nullptr;
    int *dev_err = nullptr;   // device-side bounded-wait failures
    double *logp1 = nullptr, *logp2 = nullptr;
    float *bfit_init1 = nullptr, *bfit_init2 = nullptr, *bfit_par = nullptr, *bfit_chi2 = nullptr,
          *bfit_hess = nullptr, *bfit_res = nullptr;
    int *bfit_state = nullptr, *bfit_iter = nullptr;
    // internal copies of outputs the fit needs
    double *acf_int = nullptr, *var_int = nullptr;
    // surrogate-seeded fits (allocated when a surrogate is first attached)
    imfcs_surrogate *sur = nullptr;
    int sur_mode = 0;
    float *sur_x = nullptr, *sur_pred = nullptr, *sur_init = nullptr, *plain_par = nullptr, *plain_chi2 = nullptr;
    int *plain_state = nullptr, *sur_todo = nullptr, *sur_count = nullptr;
    int *lm_counter = nullptr;   // LM work counter (dynamic fit scheduling)
    int *bg_sums = nullptr;      // per-trace background sums [2][ntrace] (background image)
    bool nb_only = false;        // N&B mode of the reference calcACF: lag 1 only
    double *nb_sum = nullptr;    // its lag-1 product sums [npix]
    // host path buffers: the device stack (and, for the asynchronous host
    // path, a second one: the copy of the next stack overlaps the current
    // execution), the copy stream and the events ordering the two
    uint16_t *dstack = nullptr, *dstack2 = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copied[2] = {}, consumed[2] = {};
    int ring = 0;
    imfcs_outputs dout;
    bool dout_alloc = false;
    // stage timing
    static constexpr int kStages = 6;
    bool timing = false;
    cudaEvent_t ev[kStages + 1] = {};
    bool ev_used[kStages + 1] = {};
    ~imfcs_plan()
    {
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        for (auto &b : bufs) cudaFree(b.p);
        if (own_arena) cudaFree(own_arena);
        if (li_dev) cudaFree(li_dev);
        for (int i = 0; i <= kStages; i++)
            if (ev[i]) cudaEventDestroy(ev[i]);
        for (int i = 0; i < 2; i++) {
            if (copied[i]) cudaEventDestroy(copied[i]);
            if (consumed[i]) cudaEventDestroy(consumed[i]);
        }
        if (copy_stream) cudaStreamDestroy(copy_stream);
    }
    void mark(int i, cudaStream_t s)
    {
        if (!timing) return;
        cudaEventRecord(ev[i], s);
        ev_used[i] = true;
    }
    // per-execution scratch: one arena, owned by the plan or bound by a
    // batch that runs several plans' executions one after another on it
    struct ScratchField {
        void **ptr;
        size_t bytes;
    };
    std::vector<ScratchField> scratch;
    size_t scratch_need = 0;
    void *own_arena = nullptr;
    template <class T>
    void reserve(T *&ptr, size_t count)
    {
        size_t n = count * sizeof(T);
        n = ((n ? n : 16) + 255) & ~(size_t)255;
        scratch.push_back({reinterpret_cast<void **>(&ptr), n});
        scratch_need += n;
    }
    void bind_scratch(void *base)
    {
        size_t off = 0;
        for (auto &f : scratch) {
            *f.ptr = base ? (void *)((char *)base + off) : nullptr;
            off += f.bytes;
        }
    }
    template <class T>
    cudaError_t alloc(T *&ptr, size_t count)
    {
        void *p = nullptr;
        size_t n = count * sizeof(T);
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) return e;
        bufs.push_back({p, n});
        bytes += n;
        ptr = (T *)p;
        return cudaSuccess;
    }
};

static ModelConst model_const_from(const double *cst)
{
    ModelConst m;
    m.ax = (float)(cst[0] * 1e6); m.ay = (float)(cst[1] * 1e6);
    m.s = (float)(cst[2] * 1e6); m.sz = (float)(cst[3] * 1e6);
    m.rx = (float)(cst[4] * 1e6); m.ry = (float)(cst[5] * 1e6);
    double fo = cst[6] * 1e12;
    double ax = cst[0] * 1e6, ay = cst[1] * 1e6;
    m.inv_norm = (float)(fo / (4.0 * ax * ay * ax * ay));
    m.q2 = (float)cst[7]; m.q3 = (float)cst[8];
    return m;
}

static bool validate_config(const imfcs_config *c, std::string &err)
{
    if (!c) { err = "null config"; return false; }
    if (c->width <= 0 || c->height <= 0 || c->frames <= 0) { err = "invalid stack geometry"; return false; }
    if (c->first < 0 || c->num <= 0 || c->first + c->num > c->frames) { err = "invalid frame range"; return false; }
    if (c->out_w <= 0 || c->out_h <= 0) { err = "invalid output grid"; return false; }
    if (c->binx <= 0 || c->biny <= 0 || c->pixbinx <= 0 || c->pixbiny <= 0) { err = "invalid binning"; return false; }
    if (c->map_x0 < 0 || c->map_y0 < 0) { err = "invalid map offset"; return false; }
    // both windows of every output pixel inside the frame
    long xmin = (long)c->map_x0 * c->pixbinx, ymin = (long)c->map_y0 * c->pixbiny;
    long xmax = (long)(c->map_x0 + c->out_w - 1) * c->pixbinx + c->binx - 1;
    long ymax = (long)(c->map_y0 + c->out_h - 1) * c->pixbiny + c->biny - 1;
    if (xmin + std::min(0, c->cfx) < 0 || ymin + std::min(0, c->cfy) < 0 ||
        xmax + std::max(0, c->cfx) >= c->width || ymax + std::max(0, c->cfy) >= c->height) {
        err = "pixel windows outside the image (check binning, map offset and cf distance)";
        return false;
    }
    if (c->background < 0) { err = "Invalid background value"; return false; }
    if (c->bleach < 0 || c->bleach > 3) { err = "invalid bleach mode"; return false; }
    if (c->bleach == IMFCS_BLEACH_POLYNOMIAL && (c->poly_order < 1 || c->poly_order > kMaxPoly)) {
        err = "polynomial order must be in 1..8";
        return false;
    }
    if (!(c->frametime > 0)) { err = "invalid frame time"; return false; }
    // the GLS covariance and whitened fit hold the (chanum-1)^2 covariance
    // and L^-1 of a pixel in one CTA's shared memory: P = 16 (chanum <= 97)
    if (c->gls && c->p + (c->q - 1) * c->p / 2 > 96) {
        err = "GLS needs at most 96 fit lags (correlator P = 16)";
        return false;
    }
    return true;
}

namespace imfcs {
bool config_valid(const imfcs_config *c, std::string &err) { return validate_config(c, err); }

int plan_create_ex(const imfcs_config *cfg, int input_float, int in_w, int in_h, bool given_bleach,
                   imfcs_plan **plan_out, bool external_scratch)
{
    std::string err;
    if (!plan_out) { set_error("null plan pointer"); return 1; }
    *plan_out = nullptr;
    if (!validate_config(cfg, err)) { set_error(err); return 1; }
    imfcs_plan *pl = new imfcs_plan();
    pl->cfg = *cfg;
    int blocknum = 0;
    if (!build_lag_info(cfg->p, cfg->q, cfg->num, pl->li, pl->chanum, blocknum, err)) {
        set_error(err);
        delete pl;
        return 1;
    }
    const int chanum = pl->chanum;
    Job &j = pl->job;
    memset(&j, 0, sizeof(j));
    j.in_w = in_w; j.in_h = in_h; j.input_float = input_float;
    pl->given_bleach = given_bleach;
    j.first = cfg->first; j.num = cfg->num;
    j.out_w = cfg->out_w; j.out_h = cfg->out_h; j.map_x0 = cfg->map_x0; j.map_y0 = cfg->map_y0;
    j.binx = cfg->binx; j.biny = cfg->biny; j.pixbinx = cfg->pixbinx; j.pixbiny = cfg->pixbiny;
    j.cfx = cfg->cfx; j.cfy = cfg->cfy; j.background = cfg->background;
    j.is_ccf = (cfg->cfx != 0 || cfg->cfy != 0);
    j.npix = cfg->out_w * cfg->out_h;
    j.ntrace = j.npix * (j.is_ccf ? 2 : 1);
    j.p = cfg->p; j.q = cfg->q; j.chanum = chanum;
    j.nopit = cfg->num < 1000 ? cfg->num : 1000;
    j.ave = (int)floor((double)cfg->num / j.nopit);
    j.frametime = (float)cfg->frametime; j.frametime_d = cfg->frametime;
    j.bleach = cfg->bleach; j.poly_order = cfg->bleach == IMFCS_BLEACH_POLYNOMIAL ? cfg->poly_order : 0;
    j.blocknum = blocknum;
    j.nsnap = pl->li.nsnap;
    pl->npix = j.npix;
    pl->nseg = (cfg->num + kSeg - 1) / kSeg;
    pl->nbseg = (cfg->num - 1 + kBlkSeg - 1) / kBlkSeg;
    pl->pnum_max = pl->li.pnum_by_ind[0];
    pl->num_sms = device_sms();
    pl->k = 0;
    for (int i = 0; i < IMFCS_NPARAM; i++)
        if (cfg->free_mask[i]) pl->idx[pl->k++] = i;
    int fs = cfg->fitstart, fe = cfg->fitend;
    if (fs < 1) fs = 1;
    if (fe >= chanum || fe < fs) fe = chanum - 1;
    pl->cfg.fitstart = fs;
    pl->cfg.fitend = fe;
    pl->nfitpts = cfg->gls ? chanum - 1 : fe - fs + 1;
    if (cfg->max_iter <= 0) pl->cfg.max_iter = 2000;

    cudaError_t e = cudaSuccess;
    const size_t nt = j.ntrace, np = j.npix;
#define AL(ptr, n) if (e == cudaSuccess) e = pl->alloc(ptr, (size_t)(n))
#define AS(ptr, n) pl->reserve(ptr, (size_t)(n))
    e = cudaMalloc(&pl->li_dev, sizeof(LagInfo));   // freed separately in the destructor
    if (e != cudaSuccess) pl->li_dev = nullptr;
    AS(pl->trace, nt * j.nopit);
    AS(pl->bparams, nt * kBleachStride);
    AL(pl->snap_pos, kMaxSnap);
    AS(pl->segtot, nt * pl->nseg);
    AS(pl->snap_part, nt * j.nsnap);
    AS(pl->segbad, nt * pl->nseg);
    AS(pl->snap_bad, nt * j.nsnap);
    AS(pl->mon, np * chanum);
    AS(pl->blkmon, np);
    AS(pl->s1, np * pl->nbseg * (kBlkSegLog + 1));
    AS(pl->s2, np * pl->nbseg * (kBlkSegLog + 1));
    AS(pl->segsum, np * pl->nbseg);
    AS(pl->blk_ind, np);
    AS(pl->blk_ok, np);
    AS(pl->stats, corr_stats_floats(j));
    AS(pl->streams, corr_stream_floats(j));
    AS(pl->s0, level0_stream_floats(j));
    AS(pl->acf_int, np * chanum);
    AS(pl->var_int, np * chanum);
    AL(pl->lagtime, chanum);
    AL(pl->dev_err, 1);
    if (j.bleach == IMFCS_BLEACH_POLYNOMIAL) {
        AL(pl->proj, (size_t)(j.poly_order + 1) * j.nopit);
        AL(pl->basis, (size_t)(j.poly_order + 1) * j.num);
    }
    if (cfg->gls) {
        AS(pl->bprod, np * (chanum - 1) * (size_t)pl->pnum_max);
        AS(pl->linv, np * (size_t)(chanum - 1) * chanum / 2);
        AS(pl->ytrans, np * (chanum - 1));
        AS(pl->gls_ok, np);
    }
    if (cfg->do_fit || cfg->bayes) {
        AS(pl->fit_y, np * pl->nfitpts);
        AS(pl->fit_w, np * pl->nfitpts);
        AL(pl->fit_x, pl->nfitpts);
        AL(pl->fit_init, IMFCS_NPARAM);
        AS(pl->fit_par, np * IMFCS_NPARAM);
        AS(pl->fit_chi2, np);
        AS(pl->fit_hess, np * IMFCS_NPARAM * IMFCS_NPARAM);
        AS(pl->fit_state, np);
        AS(pl->fit_iter, np);
        AL(pl->lm_counter, 1);
    }
    if (cfg->bayes) {
        AS(pl->logp1, np);
        AS(pl->logp2, np);
        AL(pl->bfit_init1, IMFCS_NPARAM);
        AL(pl->bfit_init2, IMFCS_NPARAM);
        AS(pl->bfit_res, np * IMFCS_NPARAM);
    }
#undef AL
#undef AS
    // the scratch arena (a batch binds its own instead)
    if (e == cudaSuccess && !external_scratch) {
        e = cudaMalloc(&pl->own_arena, pl->scratch_need);
        if (e != cudaSuccess) pl->own_arena = nullptr;
        else {
            pl->bytes += pl->scratch_need;
            pl->bind_scratch(pl->own_arena);
        }
    }
    if (e != cudaSuccess) {
        set_error(cuda_msg(e, "plan allocation"));
        delete pl;
        return 1;
    }
    // constant tables
    e = cudaMemcpy(pl->li_dev, &pl->li, sizeof(LagInfo), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(pl->dev_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(pl->snap_pos, pl->li.snap_pos, sizeof(int) * kMaxSnap, cudaMemcpyHostToDevice);
    std::vector<float> lt(chanum);
    for (int x = 0; x < chanum; x++) lt[x] = (float)(pl->li.lag[x] * cfg->frametime);
    if (e == cudaSuccess) e = cudaMemcpy(pl->lagtime, lt.data(), sizeof(float) * chanum, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && j.bleach == IMFCS_BLEACH_POLYNOMIAL) {
        std::vector<double> proj((size_t)(j.poly_order + 1) * j.nopit);
        legendre_projection(j.poly_order, j.nopit, j.ave, cfg->frametime, proj.data(), pl->uscale, pl->uoff);
        std::vector<float> table((size_t)(j.poly_order + 1) * j.num);
        legendre_basis_table(j.poly_order, j.num, cfg->frametime, pl->uscale, pl->uoff, table.data());
        e = cudaMemcpy(pl->proj, proj.data(), proj.size() * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(pl->basis, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && (cfg->do_fit || cfg->bayes)) {
        std::vector<float> xs(pl->nfitpts), init(IMFCS_NPARAM);
        int off = cfg->gls ? 1 : pl->cfg.fitstart;
        for (int i = 0; i < pl->nfitpts; i++) xs[i] = lt[off + i];
        for (int i = 0; i < IMFCS_NPARAM; i++) init[i] = (float)(cfg->init[i] / param_unit(i));
        e = cudaMemcpy(pl->fit_x, xs.data(), sizeof(float) * pl->nfitpts, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(pl->fit_init, init.data(), sizeof(float) * IMFCS_NPARAM, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && cfg->bayes) {
            // bayesFit initial values (java:10127-10156, 10191-10220)
            std::vector<float> i1(IMFCS_NPARAM, 0.f), i2(IMFCS_NPARAM, 0.f);
            i1[0] = init[0]; i1[1] = init[1]; i1[4] = init[4];
            i2 = i1;
            i2[5] = 0.5f;
            i2[6] = (float)(0.1 * cfg->init[1] / param_unit(6));
            e = cudaMemcpy(pl->bfit_init1, i1.data(), sizeof(float) * IMFCS_NPARAM, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(pl->bfit_init2, i2.data(), sizeof(float) * IMFCS_NPARAM, cudaMemcpyHostToDevice);
        }
    }
    if (e != cudaSuccess) {
        set_error(cuda_msg(e, "plan set-up"));
        delete pl;
        return 1;
    }
    memset(&pl->dout, 0, sizeof(pl->dout));
    *plan_out = pl;
    return 0;
}
}  // namespace imfcs

extern "C" int imfcs_plan_create(const imfcs_config *cfg, imfcs_plan **plan_out)
{
    if (!cfg) { set_error("null config"); return 1; }
    return plan_create_ex(cfg, 0, cfg->width, cfg->height, false, plan_out);
}

extern "C" int imfcs_plan_destroy(imfcs_plan *plan)
{
    delete plan;
    return 0;
}

extern "C" size_t imfcs_plan_scratch_bytes(const imfcs_plan *plan) { return plan ? plan->bytes : 0; }

// One LM pass over the plan's pixels (those with todo[pix] != 0 when todo is
// given), from init[pix * init_stride] (internal units).
struct LMOut {
    float *par, *chi2, *hess;
    int *state, *iters;
};
static int run_lm(imfcs_plan *pl, cudaStream_t s, const float *y, const float *w, const float *init,
                  int init_stride, int k, const int *idx, const int *todo, const LMOut &o)
{
    const imfcs_config &c = pl->cfg;
    FitArgs a;
    memset(&a, 0, sizeof(a));
    a.nfits = pl->npix;
    a.npts = pl->nfitpts;
    a.model = IMFCS_MODEL_ACF_1D;
    a.np = IMFCS_NPARAM;
    a.k = k;
    for (int i = 0; i < k; i++) a.idx[i] = idx[i];
    a.max_iter = c.max_iter;
    a.tol = 0.f;
    a.y = y;
    a.w = w;
    a.x = pl->fit_x;
    a.init = init;
    a.init_stride = init_stride;
    a.cst = nullptr;
    a.mc = model_const_from(c.cst);
    a.linv = c.gls ? pl->linv : nullptr;
    a.out_par = o.par;
    a.out_stride = IMFCS_NPARAM;
    a.out_chi2 = o.chi2;
    a.out_state = o.state;
    a.out_iter = o.iters;
    a.out_hess = o.hess;
    a.todo = todo;
    a.counter = pl->lm_counter;
    // held flow, second/third component and triplet fractions all zero: the
    // default one-component model (seeds change only N, D, G)
    a.tirf_zero_held = c.init[2] == 0 && c.init[3] == 0 && c.init[5] == 0 && c.init[7] == 0 && c.init[9] == 0;
    CK(launch_lm(a, pl->num_sms, s));
    pl->launches += 1;
    return 0;
}

// The fit epilogue over the LM results in par_scratch / fit_chi2 /
// fit_state / fit_hess: SI parameters, reduced chi^2, fitted flags, Bayes
// terms.
static int run_epilogue(imfcs_plan *pl, cudaStream_t s, const double *acf, int k, const int *idx,
                        float *fitres, float *chi2, int *fitted, double *logp, const float *par_scratch)
{
    const imfcs_config &c = pl->cfg;
    EpilogueArgs e;
    memset(&e, 0, sizeof(e));
    e.npix = pl->npix;
    e.chanum = pl->chanum;
    e.npts = pl->nfitpts;
    e.k = k;
    for (int i = 0; i < k; i++) e.idx[i] = idx[i];
    e.fitstart = c.fitstart;
    e.fitend = c.fitend;
    e.gls = c.gls;
    e.chi2_div = c.gls ? (double)(pl->chanum - k - 1) : (double)((c.fitend - c.fitstart) - k - 1);
    e.par_int = par_scratch;
    e.chi2_raw = pl->fit_chi2;
    e.state = pl->fit_state;
    e.hess = pl->fit_hess;
    e.fitres = fitres;
    e.chi2 = chi2;
    e.fitted = fitted;
    e.logp = logp;
    e.pre_ok = c.gls ? pl->gls_ok : nullptr;
    e.acf = acf;
    e.linv = pl->linv;
    e.mc = model_const_from(c.cst);
    e.lagtime = pl->lagtime;
    CK(launch_fit_epilogue(e, s));
    pl->launches += 1;
    return 0;
}

// Plain LM from the shared initial values plus the epilogue.
static int run_fit(imfcs_plan *pl, cudaStream_t s, const double *acf, const float *y, const float *w,
                   const float *init, int k, const int *idx, float *fitres, float *chi2, int *fitted,
                   int *iters, double *logp, float *par_scratch)
{
    const LMOut o{par_scratch, pl->fit_chi2, pl->fit_hess, pl->fit_state, iters ? iters : pl->fit_iter};
    if (run_lm(pl, s, y, w, init, 0, k, idx, nullptr, o)) return 1;
    return run_epilogue(pl, s, acf, k, idx, fitres, chi2, fitted, logp, par_scratch);
}

// Surrogate-seeded LM: features + MLP + per-pixel seeds, the seeded LM, the
// refit decision (and in mode 2 the plain-LM arbiter), LM from the configured
// initial values on the refit pixels, then the epilogue.
static int run_fit_seeded(imfcs_plan *pl, cudaStream_t s, const double *acf, const double *var, const float *y,
                          const float *w, float *fitres, float *chi2, int *fitted, int *iters)
{
    int *it_out = iters ? iters : pl->fit_iter;
    CK(cudaMemsetAsync(pl->sur_count, 0, 2 * sizeof(int), s));
    if (surrogate_seed(pl->sur, pl->npix, pl->chanum, pl->k, pl->idx, acf, var, pl->sur_x, pl->sur_pred,
                       pl->fit_init, pl->sur_init, s))
        return 1;
    pl->launches += 7;   // features, BF16 inputs, 3 GEMMs, de-standardise, seeds
    if (pl->sur_mode == 2) {
        const LMOut arbiter{pl->plain_par, pl->plain_chi2, nullptr, pl->plain_state, nullptr};
        if (run_lm(pl, s, y, w, pl->fit_init, 0, pl->k, pl->idx, nullptr, arbiter)) return 1;
    }
    const LMOut o{pl->fit_par, pl->fit_chi2, pl->fit_hess, pl->fit_state, it_out};
    if (run_lm(pl, s, y, w, pl->sur_init, IMFCS_NPARAM, pl->k, pl->idx, nullptr, o)) return 1;
    CK(launch_seed_select(pl->npix, pl->k, pl->idx, pl->fit_par, pl->fit_state, pl->fit_chi2,
                          pl->sur_mode == 2 ? pl->plain_state : nullptr, pl->sur_mode == 2 ? pl->plain_chi2 : nullptr,
                          y, w, pl->nfitpts, pl->sur_todo, pl->sur_count, s));
    pl->launches += 1;
    if (run_lm(pl, s, y, w, pl->fit_init, 0, pl->k, pl->idx, pl->sur_todo, o)) return 1;
    return run_epilogue(pl, s, acf, pl->k, pl->idx, fitres, chi2, fitted, nullptr, pl->fit_par);
}

namespace imfcs {
int fit_stage(imfcs_plan *pl, cudaStream_t s, const double *acf, const double *var, const imfcs_outputs *dev_out);

int plan_execute_any(imfcs_plan *pl, const void *dev_stack, const imfcs_outputs *dev_out, void *stream)
{
    if (!pl || !dev_stack || !dev_out) { set_error("null argument"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    const Job &j = pl->job;
    const imfcs_config &c = pl->cfg;
    const int chanum = pl->chanum;
    double *acf = dev_out->acf ? dev_out->acf : pl->acf_int;
    double *var = dev_out->var ? dev_out->var : pl->var_int;
    for (int i = 0; i <= imfcs_plan::kStages; i++) pl->ev_used[i] = false;
    pl->launches = 0;
    pl->mark(0, s);
    CK(launch_trace(j, dev_stack, pl->trace, s));
    if (pl->given_bleach) CK(launch_center_given(j, pl->trace, pl->bparams, s));
    else CK(launch_bleach(j, pl->trace, pl->proj, (float)pl->uscale, (float)pl->uoff, pl->bparams, s));
    pl->launches += 2;
    pl->mark(1, s);
    // one streaming pass over the raw stack: the corrected, centred level-0
    // stream and the monitor partial sums
    CK(launch_stream(j, dev_stack, pl->bparams, pl->basis, pl->snap_pos, pl->nseg, pl->s0, pl->segtot,
                     pl->snap_part, pl->segbad, pl->snap_bad, pl->dev_err, s));
    CK(launch_monitor_finalize(j, pl->li_dev, pl->bparams, pl->nseg, pl->segtot, pl->snap_part, pl->segbad,
                               pl->snap_bad, pl->mon, pl->blkmon, s));
    pl->launches += 2;
    pl->mark(2, s);
    if (pl->nb_only) {
        // N&B mode: lag 1 only; the correlator, blocking and fits do not run
        if (!pl->nb_sum) CK(pl->alloc(pl->nb_sum, pl->npix));
        CK(launch_nb_lag1(j, pl->s0, pl->mon, pl->nb_sum, dev_out->nb_mean, dev_out->nb_cov, s));
        pl->launches += 2;
        for (int i = 3; i <= 6; i++) pl->mark(i, s);
        return 0;
    }
    CK(launch_block(j, pl->s0, pl->blkmon, pl->nbseg, pl->s1, pl->s2, pl->segsum, pl->blk_ind, pl->blk_ok, s));
    pl->launches += 2;
    pl->mark(3, s);
    CK(launch_corr(j, pl->li_dev, dev_stack, pl->bparams, pl->basis, pl->s0, pl->mon, pl->blk_ind, acf, var,
                   dev_out->sd, dev_out->nb_mean, dev_out->nb_cov, pl->bprod, pl->pnum_max, pl->stats, pl->streams,
                   c.gls, pl->dev_err, s));
    pl->launches += corr_kernel_count(j);
    if (dev_out->blocked_ind) CK(cudaMemcpyAsync(dev_out->blocked_ind, pl->blk_ind, sizeof(int) * pl->npix, cudaMemcpyDeviceToDevice, s));
    if (dev_out->blocked_ok) CK(cudaMemcpyAsync(dev_out->blocked_ok, pl->blk_ok, sizeof(int) * pl->npix, cudaMemcpyDeviceToDevice, s));
    pl->mark(4, s);
    if (c.gls) {
        GlsArgs g;
        memset(&g, 0, sizeof(g));
        g.npix = pl->npix;
        g.chanum = chanum;
        g.pnum_stride = pl->pnum_max;
        g.bprod = pl->bprod;
        g.mon = pl->mon;
        g.blk_ind = pl->blk_ind;
        g.pnum_by_ind = (const int *)((const char *)pl->li_dev + offsetof(LagInfo, pnum_by_ind));
        g.linv = pl->linv;
        g.ytrans = pl->ytrans;
        g.ok = pl->gls_ok;
        g.covmats_out = dev_out->covmats;
        CK(launch_gls(g, s));
        pl->launches += 1;
    }
    pl->mark(5, s);
    if (fit_stage(pl, s, acf, var, dev_out)) return 1;
    pl->mark(6, s);
    return 0;
}

// The fits over the correlator outputs acf/var of the plan's last execution
// (with the plan's current model constants).
int fit_stage(imfcs_plan *pl, cudaStream_t s, const double *acf, const double *var, const imfcs_outputs *dev_out)
{
    const imfcs_config &c = pl->cfg;
    const int chanum = pl->chanum;
    if (c.do_fit || c.bayes) {
        const float *y = c.gls ? pl->ytrans : pl->fit_y;
        const float *w = c.gls ? nullptr : pl->fit_w;
        if (!c.gls) {
            CK(launch_ols_prepare(pl->npix, chanum, c.fitstart, pl->nfitpts, acf, var, pl->fit_y, pl->fit_w, s));
            pl->launches += 1;
        }
        if (c.do_fit) {
            if (!dev_out->fitres) { set_error("fitres output required when do_fit is set"); return 1; }
            if (pl->sur && pl->sur_mode) {
                if (run_fit_seeded(pl, s, acf, var, y, w, dev_out->fitres, dev_out->chi2, dev_out->fitted,
                                   dev_out->iterations))
                    return 1;
            } else if (run_fit(pl, s, acf, y, w, pl->fit_init, pl->k, pl->idx, dev_out->fitres, dev_out->chi2,
                               dev_out->fitted, dev_out->iterations, nullptr, pl->fit_par)) {
                return 1;
            }
        }
        if (c.bayes) {
            const int i1[3] = {0, 1, 4}, i2[5] = {0, 1, 4, 5, 6};
            if (run_fit(pl, s, acf, y, w, pl->bfit_init1, 3, i1, pl->bfit_res, nullptr, nullptr, nullptr,
                        pl->logp1, pl->fit_par))
                return 1;
            if (run_fit(pl, s, acf, y, w, pl->bfit_init2, 5, i2, pl->bfit_res, nullptr, nullptr, nullptr,
                        pl->logp2, pl->fit_par))
                return 1;
            if (dev_out->bayes_prob) {
                CK(launch_bayes_combine(pl->npix, pl->logp1, pl->logp2, dev_out->bayes_prob, s));
                pl->launches += 1;
            }
        }
    }
    return 0;
}
}  // namespace imfcs

extern "C" int imfcs_plan_set_surrogate(imfcs_plan *pl, imfcs_surrogate *sur, int mode)
{
    if (!pl) { set_error("null plan"); return 1; }
    if (mode < 0 || mode > 2) { set_error("surrogate mode must be 0, 1 or 2"); return 1; }
    if (!sur || mode == 0) {
        pl->sur = nullptr;
        pl->sur_mode = 0;
        return 0;
    }
    if (!pl->cfg.do_fit) { set_error("the surrogate seeds the do_fit LM: enable do_fit"); return 1; }
    if (pl->chanum < IMFCS_SURROGATE_INPUTS / 2 + 1) {
        set_error("the surrogate reads lags 1..64: the plan needs at least 65 correlation channels");
        return 1;
    }
    if (!pl->sur_x) {
        const size_t np = pl->npix;
        cudaError_t e = pl->alloc(pl->sur_x, np * IMFCS_SURROGATE_INPUTS);
        if (e == cudaSuccess) e = pl->alloc(pl->sur_pred, np * IMFCS_SURROGATE_OUTPUTS);
        if (e == cudaSuccess) e = pl->alloc(pl->sur_init, np * IMFCS_NPARAM);
        if (e == cudaSuccess) e = pl->alloc(pl->plain_par, np * IMFCS_NPARAM);
        if (e == cudaSuccess) e = pl->alloc(pl->plain_chi2, np);
        if (e == cudaSuccess) e = pl->alloc(pl->plain_state, np);
        if (e == cudaSuccess) e = pl->alloc(pl->sur_todo, np);
        if (e == cudaSuccess) e = pl->alloc(pl->sur_count, 2);
        if (e == cudaSuccess) e = cudaMemset(pl->sur_count, 0, 2 * sizeof(int));
        if (e != cudaSuccess) {
            pl->sur_x = nullptr;
            set_error(cuda_msg(e, "surrogate buffers"));
            return 1;
        }
    }
    if (surrogate_reserve(sur, pl->npix)) return 1;
    pl->sur = sur;
    pl->sur_mode = mode;
    return 0;
}

extern "C" int imfcs_plan_set_background_image(imfcs_plan *pl, const double *host_bg)
{
    if (!pl) { set_error("null plan"); return 1; }
    Job &j = pl->job;
    if (j.input_float) { set_error("the float-stack path takes background-subtracted data"); return 1; }
    if (!host_bg) {
        j.bg_trace = nullptr;
        j.bg_avg = nullptr;
        return 0;
    }
    const size_t n = (size_t)j.in_w * j.in_h;
    std::vector<int> r(n);
    for (size_t i = 0; i < n; i++) {
        const double v = host_bg[i];
        if (!std::isfinite(v) || v < -2e9 || v > 2e9) { set_error("background image holds an invalid value"); return 1; }
        r[i] = (int)std::floor(v + 0.5);   // Math.round
    }
    // per trace: its own window (values) and the direct window (averaged trace)
    std::vector<int> sums((size_t)2 * j.ntrace);
    for (int tr = 0; tr < j.ntrace; tr++) {
        int x0, y0, xd, yd;
        trace_origin(j, tr, x0, y0);
        trace_origin(j, tr % j.npix, xd, yd);
        long s = 0, sa = 0;
        for (int k = 0; k < j.biny; k++)
            for (int i = 0; i < j.binx; i++) {
                s += r[(size_t)(y0 + k) * j.in_w + x0 + i];
                sa += r[(size_t)(yd + k) * j.in_w + xd + i];
            }
        sums[tr] = (int)s;
        sums[(size_t)j.ntrace + tr] = (int)sa;
    }
    if (!pl->bg_sums) {
        cudaError_t e = pl->alloc(pl->bg_sums, sums.size());
        if (e != cudaSuccess) { set_error(cuda_msg(e, "background image buffer")); return 1; }
    }
    CK(cudaMemcpy(pl->bg_sums, sums.data(), sums.size() * sizeof(int), cudaMemcpyHostToDevice));
    j.bg_trace = pl->bg_sums;
    j.bg_avg = pl->bg_sums + j.ntrace;
    return 0;
}

extern "C" int imfcs_plan_surrogate_stats(const imfcs_plan *pl, int *n_refit, int *n_worse)
{
    if (!pl) { set_error("null plan"); return 1; }
    int c[2] = {0, 0};
    if (pl->sur_count) CK(cudaMemcpy(c, pl->sur_count, sizeof(c), cudaMemcpyDeviceToHost));
    if (n_refit) *n_refit = c[0];
    if (n_worse) *n_worse = c[1];
    return 0;
}

extern "C" int imfcs_plan_execute(imfcs_plan *pl, const uint16_t *dev_stack,
                                  const imfcs_outputs *dev_out, void *stream)
{
    return plan_execute_any(pl, dev_stack, dev_out, stream);
}

template <class T>
static cudaError_t d2h(T *host, const T *dev, size_t n, cudaStream_t s)
{
    if (!host || !dev) return cudaSuccess;
    return cudaMemcpyAsync(host, dev, n * sizeof(T), cudaMemcpyDeviceToHost, s);
}

// Enqueues one host-buffer execution on `s`: the stack copy on the plan's
// copy stream into buffer `b` (after the execution that last read that
// buffer), the execution after the copy, the results' copies after the
// execution.  Returns without synchronising.
static int execute_host_enqueue(imfcs_plan *pl, const uint16_t *host_stack, const imfcs_outputs *host_out,
                                cudaStream_t s, int b)
{
    const imfcs_config &c = pl->cfg;
    const size_t np = pl->npix, ch = pl->chanum;
    const size_t fsz = (size_t)c.width * c.height;
    uint16_t *&buf = b ? pl->dstack2 : pl->dstack;
    if (!buf) {
        uint16_t *p = nullptr;
        cudaError_t e = pl->alloc(p, fsz * c.frames);
        if (e != cudaSuccess) { set_error(cuda_msg(e, "stack allocation")); return 1; }
        buf = p;
    }
    if (!pl->copy_stream) {
        CK(cudaStreamCreateWithFlags(&pl->copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; i++) {
            CK(cudaEventCreateWithFlags(&pl->copied[i], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&pl->consumed[i], cudaEventDisableTiming));
        }
    }
    if (!pl->dout_alloc) {
        imfcs_outputs &d = pl->dout;
        cudaError_t e = cudaSuccess;
#define OA(field, n) if (e == cudaSuccess && host_out->field) e = pl->alloc(d.field, (size_t)(n))
        OA(acf, np * ch); OA(var, np * ch); OA(sd, np * ch);
        OA(blocked_ind, np); OA(blocked_ok, np); OA(nb_mean, np); OA(nb_cov, np);
        OA(fitres, np * IMFCS_NPARAM); OA(chi2, np); OA(fitted, np); OA(iterations, np);
        OA(bayes_prob, np * 2); OA(covmats, np * (ch - 1) * (ch - 1));
#undef OA
        if (e != cudaSuccess) { set_error(cuda_msg(e, "output allocation")); return 1; }
        pl->dout_alloc = true;
    }
    // only the frames the job reads
    CK(cudaStreamWaitEvent(pl->copy_stream, pl->consumed[b], 0));
    CK(cudaMemcpyAsync(buf + fsz * c.first, host_stack + fsz * c.first, fsz * c.num * sizeof(uint16_t),
                       cudaMemcpyHostToDevice, pl->copy_stream));
    CK(cudaEventRecord(pl->copied[b], pl->copy_stream));
    CK(cudaStreamWaitEvent(s, pl->copied[b], 0));
    if (imfcs_plan_execute(pl, buf, &pl->dout, s)) return 1;
    CK(cudaEventRecord(pl->consumed[b], s));
    const imfcs_outputs &d = pl->dout;
    CK(d2h(host_out->acf, d.acf, np * ch, s));
    CK(d2h(host_out->var, d.var, np * ch, s));
    CK(d2h(host_out->sd, d.sd, np * ch, s));
    CK(d2h(host_out->blocked_ind, d.blocked_ind, np, s));
    CK(d2h(host_out->blocked_ok, d.blocked_ok, np, s));
    CK(d2h(host_out->nb_mean, d.nb_mean, np, s));
    CK(d2h(host_out->nb_cov, d.nb_cov, np, s));
    CK(d2h(host_out->fitres, d.fitres, np * IMFCS_NPARAM, s));
    CK(d2h(host_out->chi2, d.chi2, np, s));
    CK(d2h(host_out->fitted, d.fitted, np, s));
    CK(d2h(host_out->iterations, d.iterations, np, s));
    CK(d2h(host_out->bayes_prob, d.bayes_prob, np * 2, s));
    CK(d2h(host_out->covmats, d.covmats, np * (ch - 1) * (ch - 1), s));
    return 0;
}

extern "C" int imfcs_plan_synchronize(imfcs_plan *pl, void *stream)
{
    if (!pl) { set_error("null plan"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    int derr = 0;
    CK(cudaMemcpyAsync(&derr, pl->dev_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (derr) { set_error("a device-side wait timed out (TMA staging)"); return 1; }
    return 0;
}

extern "C" int imfcs_plan_execute_host(imfcs_plan *pl, const uint16_t *host_stack,
                                       const imfcs_outputs *host_out, void *stream)
{
    if (!pl || !host_stack || !host_out) { set_error("null argument"); return 1; }
    if (execute_host_enqueue(pl, host_stack, host_out, (cudaStream_t)stream, 0)) return 1;
    return imfcs_plan_synchronize(pl, stream);
}

extern "C" int imfcs_plan_execute_host_async(imfcs_plan *pl, const uint16_t *host_stack,
                                             const imfcs_outputs *host_out, void *stream)
{
    if (!pl || !host_stack || !host_out) { set_error("null argument"); return 1; }
    const int b = pl->ring;
    pl->ring ^= 1;
    return execute_host_enqueue(pl, host_stack, host_out, (cudaStream_t)stream, b);
}

namespace imfcs {
float *plan_bparams(imfcs_plan *pl) { return pl->bparams; }
const Job &plan_job(imfcs_plan *pl) { return pl->job; }
void plan_set_nb_only(imfcs_plan *pl, bool on) { pl->nb_only = on; }
void plan_umap(imfcs_plan *pl, double &uscale, double &uoff)
{
    // u-mapping of the averaged-trace time axis (same as legendre_projection)
    const Job &j = pl->job;
    double t0 = j.frametime_d * 0.5 * j.ave, t1 = j.frametime_d * (j.nopit - 0.5) * j.ave;
    uscale = (t1 > t0) ? 2.0 / (t1 - t0) : 1.0;
    uoff = -1.0 - t0 * uscale;
}
const LagInfo &plan_laginfo(imfcs_plan *pl) { return pl->li; }
}  // namespace imfcs

// ---------------------------------------------------------------------------
// FCS diffusion law (dlfit java:11007-11231, determineDiffusionLaw
// 8190-8250, fitDiffLaw 8253-8295, LineFit 10792-10842), "All" non-overlap
// mode: binning u = n_bin..1, output grid floor(W/u) x floor(H/u) at pixel
// stride u, one-component fit of every pixel, mean and variance of D over
// the fitted pixels.
// ---------------------------------------------------------------------------
__global__ void dl_reduce_kernel(int npix, const float *fitres, const int *fitted, double *acc)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double c = 0, s = 0, s2 = 0;
    if (i < npix && fitted[i]) {
        double d = fitres[(size_t)i * IMFCS_NPARAM + 1];
        c = 1;
        s = d;
        s2 = d * d;
    }
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_xor_sync(0xffffffffu, c, o);
        s += __shfl_xor_sync(0xffffffffu, s, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], c);
        atomicAdd(&acc[1], s);
        atomicAdd(&acc[2], s2);
    }
}

static double obsvol_2d_host(double ax, double ay, double s)
{
    const double sqrpi = sqrt(3.14159265359);
    double px = s / sqrpi * (2 * exp(-(ax / s) * (ax / s)) - 2) + 2 * ax * erf(ax / s);
    double py = s / sqrpi * (2 * exp(-(ay / s) * (ay / s)) - 2) + 2 * ay * erf(ay / s);
    return 4 * (ax * ay) * (ax * ay) / (px * py);
}

extern "C" int imfcs_diffusion_law(const imfcs_config *cfg, const uint16_t *dev_stack, int n_bin,
                                   int fit_lo, int fit_hi, double pixel_size_m, double psf_m,
                                   double *out, double *line, void *stream)
{
    if (!cfg || !dev_stack || !out || n_bin < 1) { set_error("invalid argument"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    double *acc = nullptr;
    CK(cudaMalloc(&acc, 3 * sizeof(double)));
    int rc = 0;
    for (int u = n_bin; u >= 1 && rc == 0; u--) {
        imfcs_config c = *cfg;
        c.binx = c.biny = c.pixbinx = c.pixbiny = u;
        c.map_x0 = c.map_y0 = 0;
        c.out_w = c.width / u;
        c.out_h = c.height / u;
        c.cfx = c.cfy = 0;
        c.do_fit = 1;
        c.bayes = 0;
        const double ax = pixel_size_m * u, ay = pixel_size_m * u;
        c.cst[0] = ax; c.cst[1] = ay; c.cst[2] = psf_m; c.cst[4] = 0; c.cst[5] = 0;
        c.cst[6] = obsvol_2d_host(ax, ay, psf_m);
        imfcs_plan *pl = nullptr;
        if (imfcs_plan_create(&c, &pl)) { rc = 1; break; }
        const int np = pl->npix;
        float *fitres = nullptr, *chi2 = nullptr;
        int *fitted = nullptr;
        cudaError_t e = cudaMalloc(&fitres, sizeof(float) * np * IMFCS_NPARAM);
        if (e == cudaSuccess) e = cudaMalloc(&chi2, sizeof(float) * np);
        if (e == cudaSuccess) e = cudaMalloc(&fitted, sizeof(int) * np);
        imfcs_outputs o;
        memset(&o, 0, sizeof(o));
        o.fitres = fitres; o.chi2 = chi2; o.fitted = fitted;
        double h[3] = {0, 0, 0};
        if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, 3 * sizeof(double), s);
        if (e != cudaSuccess) { set_error(cuda_msg(e, "diffusion-law buffers")); rc = 1; }
        if (!rc && imfcs_plan_execute(pl, dev_stack, &o, stream)) rc = 1;
        if (!rc) {
            dl_reduce_kernel<<<(np + 255) / 256, 256, 0, s>>>(np, fitres, fitted, acc);
            e = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) { set_error(cuda_msg(e, "diffusion-law reduction")); rc = 1; }
        }
        if (!rc) {
            double aeff = obsvol_2d_host(ax, ay, psf_m) * 1e12;      // um^2 (java:11139)
            double meanD = h[1] * 1e12 / h[0];                        // java:11189-11191
            double varD = h[2] * 1e24 / h[0] - meanD * meanD;
            out[3 * (u - 1) + 0] = aeff;
            out[3 * (u - 1) + 1] = meanD;
            out[3 * (u - 1) + 2] = varD;
        }
        cudaFree(fitres);
        cudaFree(chi2);
        cudaFree(fitted);
        imfcs_plan_destroy(pl);
    }
    cudaFree(acc);
    if (rc) return 1;
    if (line) {
        // fitDiffLaw: y = Aeff/D, sd = Aeff/D^2 sqrt(var D) (java:8207-8210), weighted line
        int lo = fit_lo - 1, hi = fit_hi - 1;
        if (lo < 0 || hi >= n_bin || lo >= hi) { set_error("Fit start/end not correctly set."); return 1; }
        double sw = 0, sx = 0, sy = 0, sxx = 0, sxy = 0;
        for (int i = lo; i <= hi; i++) {
            double x = out[3 * i], D = out[3 * i + 1], v = out[3 * i + 2];
            double y = x / D, sd = x / (D * D) * sqrt(v);
            double w = 1.0 / (sd * sd);
            sw += w; sx += w * x; sy += w * y; sxx += w * x * x; sxy += w * x * y;
        }
        double det = sw * sxx - sx * sx;
        line[1] = (sw * sxy - sx * sy) / det;
        line[0] = (sy - line[1] * sx) / sw;
    }
    return 0;
}

extern "C" int imfcs_psf_calibration(const imfcs_config *cfg, const uint16_t *dev_stack, int n_bin, int bin_start,
                                     const double *psf_m, int psf_count, double pixel_size_m, double *out,
                                     void *stream)
{
    if (!cfg || !dev_stack || !out || !psf_m || n_bin < 1) { set_error("invalid argument"); return 1; }
    if (cfg->width < 20 || cfg->height < 20) {
        set_error("Image is too small to provide good PSF statistics. At least 20x20 pixels are required.");
        return 1;
    }
    if (psf_count < 1 || psf_count >= 10) {
        set_error("PSF range and stepsize lead to too many calculations. Please chose a smaller range.");
        return 1;
    }
    cudaStream_t s = (cudaStream_t)stream;
    double *acc = nullptr;
    CK(cudaMalloc(&acc, 3 * sizeof(double)));
    int rc = 0;
    for (int u = n_bin; u >= 1 && rc == 0; u--) {
        imfcs_config c = *cfg;
        c.binx = c.biny = c.pixbinx = c.pixbiny = u;
        c.map_x0 = c.map_y0 = 0;
        c.out_w = c.width / u;
        c.out_h = c.height / u;
        c.cfx = c.cfy = 0;
        c.do_fit = 1;
        c.bayes = 0;
        const double ax = pixel_size_m * u, ay = pixel_size_m * u;
        c.cst[0] = ax; c.cst[1] = ay; c.cst[2] = psf_m[0]; c.cst[4] = 0; c.cst[5] = 0;
        c.cst[6] = obsvol_2d_host(ax, ay, psf_m[0]);
        imfcs_plan *pl = nullptr;
        if (imfcs_plan_create(&c, &pl)) { rc = 1; break; }
        const int np = pl->npix, ch = pl->chanum;
        double *acf = nullptr, *var = nullptr;
        float *fitres = nullptr, *chi2 = nullptr;
        int *fitted = nullptr;
        cudaError_t e = cudaMalloc(&acf, sizeof(double) * np * ch);
        if (e == cudaSuccess) e = cudaMalloc(&var, sizeof(double) * np * ch);
        if (e == cudaSuccess) e = cudaMalloc(&fitres, sizeof(float) * np * IMFCS_NPARAM);
        if (e == cudaSuccess) e = cudaMalloc(&chi2, sizeof(float) * np);
        if (e == cudaSuccess) e = cudaMalloc(&fitted, sizeof(int) * np);
        if (e != cudaSuccess) { set_error(cuda_msg(e, "PSF calibration buffers")); rc = 1; }
        imfcs_outputs o;
        memset(&o, 0, sizeof(o));
        o.acf = acf; o.var = var; o.fitres = fitres; o.chi2 = chi2; o.fitted = fitted;
        // the correlations once per binning; the fits for every PSF size
        if (!rc && imfcs_plan_execute(pl, dev_stack, &o, stream)) rc = 1;
        for (int ip = 0; ip < psf_count && !rc; ip++) {
            if (ip > 0) {
                pl->cfg.cst[2] = psf_m[ip];
                pl->cfg.cst[6] = obsvol_2d_host(ax, ay, psf_m[ip]);
                if (fit_stage(pl, s, acf, var, &o)) { rc = 1; break; }
            }
            double h[3] = {0, 0, 0};
            e = cudaMemsetAsync(acc, 0, 3 * sizeof(double), s);
            if (e == cudaSuccess) {
                dl_reduce_kernel<<<(np + 255) / 256, 256, 0, s>>>(np, fitres, fitted, acc);
                e = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s);
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) { set_error(cuda_msg(e, "PSF calibration reduction")); rc = 1; break; }
            // determinePSF (java:8141-8146): label u + psfBinStart for binning
            // u + 1 (0-based u), mean D, and the variance of D over
            // sqrt(width / (u + 1) * height / (u + 1)) in Java int arithmetic
            const double meanD = h[1] * 1e12 / h[0];
            const double varD = h[2] * 1e24 / h[0] - meanD * meanD;
            const int ui = u - 1;
            const int cnt = cfg->width / (ui + 1) * cfg->height / (ui + 1);
            out[((size_t)ip * 3 + 0) * n_bin + ui] = ui + bin_start;
            out[((size_t)ip * 3 + 1) * n_bin + ui] = meanD;
            out[((size_t)ip * 3 + 2) * n_bin + ui] = varD / sqrt((double)cnt);
        }
        cudaFree(acf);
        cudaFree(var);
        cudaFree(fitres);
        cudaFree(chi2);
        cudaFree(fitted);
        imfcs_plan_destroy(pl);
    }
    cudaFree(acc);
    return rc;
}

extern "C" int imfcs_plan_bleach_params(const imfcs_plan *plan, float *host_out, int max_traces)
{
    if (!plan || !host_out) { set_error("null argument"); return -1; }
    int n = plan->job.ntrace < max_traces ? plan->job.ntrace : max_traces;
    cudaError_t e = cudaMemcpy(host_out, plan->bparams, sizeof(float) * kBleachStride * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "bleach params")); return -1; }
    return n;
}

extern "C" int imfcs_plan_kernel_launches(const imfcs_plan *plan)
{
    if (!plan) { set_error("null plan"); return -1; }
    return plan->launches;
}

extern "C" int imfcs_plan_set_timing(imfcs_plan *plan, int enable)
{
    if (!plan) { set_error("null plan"); return 1; }
    if (enable && !plan->ev[0])
        for (int i = 0; i <= imfcs_plan::kStages; i++) CK(cudaEventCreate(&plan->ev[i]));
    plan->timing = enable != 0;
    return 0;
}

extern "C" int imfcs_plan_stage_times(const imfcs_plan *plan, float *ms, int max_stages)
{
    if (!plan || !ms) { set_error("null argument"); return -1; }
    int n = max_stages < imfcs_plan::kStages ? max_stages : imfcs_plan::kStages;
    for (int i = 0; i < n; i++) {
        ms[i] = 0.f;
        if (plan->ev_used[i] && plan->ev_used[i + 1]) {
            cudaError_t e = cudaEventElapsedTime(&ms[i], plan->ev[i], plan->ev[i + 1]);
            if (e != cudaSuccess) { set_error(cuda_msg(e, "cudaEventElapsedTime")); return -1; }
        }
    }
    return n;
}

// ---------------------------------------------------------------------------
// Correlator tile of the level chain and its autotuner (no counterpart in
// the reference, whose kernels use fixed 16x16 blocks, agpufitjni.cu:5521).
// ---------------------------------------------------------------------------
namespace imfcs {
size_t plan_scratch_need(const imfcs_plan *pl) { return pl->scratch_need; }
void plan_bind_scratch(imfcs_plan *pl, void *base) { pl->bind_scratch(base); }
const int *plan_dev_err(const imfcs_plan *pl) { return pl->dev_err; }

// The correlator alone over the level-0 stream, monitors and blocking of the
// plan's last execution on dev_stack (same scratch, same outputs).
int plan_corr_only(imfcs_plan *pl, const void *dev_stack, const imfcs_outputs *dev_out, cudaStream_t s)
{
    const Job &j = pl->job;
    double *acf = dev_out->acf ? dev_out->acf : pl->acf_int;
    double *var = dev_out->var ? dev_out->var : pl->var_int;
    CK(launch_corr(j, pl->li_dev, dev_stack, pl->bparams, pl->basis, pl->s0, pl->mon, pl->blk_ind, acf, var,
                   dev_out->sd, dev_out->nb_mean, dev_out->nb_cov, pl->bprod, pl->pnum_max, pl->stats, pl->streams,
                   pl->cfg.gls, pl->dev_err, s));
    return 0;
}
}  // namespace imfcs

extern "C" int imfcs_plan_set_corr_tile(imfcs_plan *pl, int cta, int seg_extra, int tail_extra)
{
    if (!pl) { set_error("null plan"); return 1; }
    if ((cta != 32 && cta != 64) || seg_extra < 0 || seg_extra > 2 || tail_extra < 0 || tail_extra > 4) {
        set_error("correlator tile: cta must be 32 or 64, seg_extra 0..2 and tail_extra 0..4");
        return 1;
    }
    pl->job.c2_cta = cta;
    pl->job.c2_seg_extra = seg_extra;
    pl->job.c2_tail_extra = tail_extra;
    return 0;
}

extern "C" int imfcs_plan_get_corr_tile(const imfcs_plan *pl, int *cta, int *seg_extra, int *tail_extra)
{
    if (!pl || !cta || !seg_extra || !tail_extra) { set_error("null argument"); return 1; }
    *cta = pl->job.c2_cta ? pl->job.c2_cta : 64;
    *seg_extra = pl->job.c2_seg_extra;
    *tail_extra = pl->job.c2_tail_extra;
    return 0;
}

extern "C" int imfcs_plan_autotune(imfcs_plan *pl, const uint16_t *dev_stack, const imfcs_outputs *dev_out,
                                   void *stream, imfcs_corr_tile *trials, int max_trials, int *n_trials)
{
    if (!pl || !dev_stack || !dev_out) { set_error("null argument"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    if (n_trials) *n_trials = 0;
    // one full execution leaves the correlator's inputs in the scratch
    const bool timing = pl->timing;
    pl->timing = false;
    int rc = plan_execute_any(pl, dev_stack, dev_out, stream);
    pl->timing = timing;
    if (rc) return 1;
    if (pl->nb_only || !corr2_supported(pl->job)) return 0;   // no chain: nothing to tune
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int n = 0;
    // median of three launches after one warm-up, of the correlator alone
    auto trial = [&](int cta, int extra, int tail, float &ms) -> int {
        pl->job.c2_cta = cta;
        pl->job.c2_seg_extra = extra;
        pl->job.c2_tail_extra = tail;
        if (plan_corr_only(pl, dev_stack, dev_out, s)) return 1;
        float t[3];
        for (int r = 0; r < 3; r++) {
            cudaError_t e = cudaEventRecord(e0, s);
            if (e == cudaSuccess && plan_corr_only(pl, dev_stack, dev_out, s)) return 1;
            if (e == cudaSuccess) e = cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t[r], e0, e1);
            if (e != cudaSuccess) { set_error(cuda_msg(e, "autotune timing")); return 1; }
        }
        std::sort(t, t + 3);
        ms = t[1];
        if (trials && n < max_trials) trials[n] = {cta, extra, tail, ms};
        n++;
        return 0;
    };
    // pixels per CTA x the pair kernels' segment (tail segment alike), then
    // the tail kernel's segment alone
    const int ctas[2] = {64, 32};
    float best = 0.f;
    int best_cta = 64, best_extra = 0, best_tail = 0;
    for (int ci = 0; ci < 2 && !rc; ci++)
        for (int xi = 0; xi < 3 && !rc; xi++) {
            float ms = 0.f;
            if (trial(ctas[ci], xi, xi, ms)) { rc = 1; break; }
            if (n == 1 || ms < best) { best = ms; best_cta = ctas[ci]; best_extra = xi; best_tail = xi; }
        }
    const int pair_extra = best_extra;
    for (int ti = 0; ti <= 4 && !rc; ti++) {
        if (ti == pair_extra) continue;
        float ms = 0.f;
        if (trial(best_cta, best_extra, ti, ms)) { rc = 1; break; }
        if (ms < best) { best = ms; best_tail = ti; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pl->job.c2_cta = best_cta;
    pl->job.c2_seg_extra = best_extra;
    pl->job.c2_tail_extra = best_tail;
    if (n_trials) *n_trials = n < max_trials ? n : max_trials;
    return rc;
}
