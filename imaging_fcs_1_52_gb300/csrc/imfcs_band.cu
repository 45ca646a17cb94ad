// imfcs_band.cu -- band-streamed execution of host stacks larger than the
// device memory a caller grants.
//
// The plugin hands the whole stack to the GPU as one float array
// (GPU_get_pixels, Imaging_FCS_1_52.java:14908-14983; agpufitjni.cu:5510,
// 5586), so a stack larger than the device's memory cannot be correlated.
// Here the job's output rows are split into bands of equal height.  Output
// pixels are independent -- every stage (trace, bleach fit, streaming pass,
// blocking, correlator, GLS, fits) works on one pixel's own windows -- so a
// band is a job of its own over the input rows its windows read: its output
// rows times the pixel step plus the halo of (binning - 1) + |cfy| rows.
//
// Bands, not frame chunks: the bleach fit needs a pixel's whole trace before
// its first corrected sample exists, and blocking needs the whole
// correlation before the variance is final, so frame chunks would read the
// host stack twice (trace pass, then correlator pass); a band reads its rows
// of the stack once.
//
// Pipeline: one plan sized for one band; two device band buffers; a copy
// stream fills one buffer (one 2D copy of the band's rows of every frame)
// while the execution stream computes the band in the other; each band's new
// output rows go back to the caller's arrays after its execution.  The last
// band is moved up to end at the last output row, so every band has the
// plan's geometry; its rows that the previous band already produced are not
// copied back (their values are the same).  A band's buffer starts at a
// whole pixel step above its first output row (m steps for a halo of
// -cfy > 0 rows above): every output window of a valid job starts at or
// below row 0 (ymin = map_y0 * pixbiny + cfy >= 0), so the first band's
// buffer starts inside the image too.
#include <string.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "imfcs_gb300.h"
#include "imfcs_host.h"

using namespace imfcs;

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) { set_error(cuda_msg(_e, #call)); return 1; } \
    } while (0)

namespace {

struct BandGeom {
    int rows = 0;      // output rows per band
    int bands = 0;
    int m = 0;         // band-local map_y0: output rows of halo above row 0, in pixel steps
    int in_rows = 0;   // input rows per band
};

BandGeom band_geom(const imfcs_config &c, int band_rows)
{
    BandGeom g;
    g.rows = std::min(std::max(band_rows, 1), c.out_h);
    g.bands = (c.out_h + g.rows - 1) / g.rows;
    const int up = std::max(0, -c.cfy);
    g.m = (up + c.pixbiny - 1) / c.pixbiny;
    g.in_rows = (g.m + g.rows - 1) * c.pixbiny + c.biny + std::max(0, c.cfy);
    return g;
}

struct BandWin {
    int out_row0;   // first output row the band computes
    int new_row0;   // first output row it adds
    int new_rows;   // rows it adds
    int in_row0;    // input row of the band buffer's row 0
};

BandWin band_win(const imfcs_config &c, const BandGeom &g, int b)
{
    BandWin w;
    w.new_row0 = b * g.rows;
    w.new_rows = std::min(g.rows, c.out_h - w.new_row0);
    w.out_row0 = std::min(w.new_row0, c.out_h - g.rows);
    w.in_row0 = (c.map_y0 + w.out_row0 - g.m) * c.pixbiny;
    return w;
}

// Per output pixel: every output an imfcs_outputs can carry.
size_t output_bytes_per_pixel(const imfcs_config &c)
{
    const size_t ch = (size_t)imfcs_chanum(c.p, c.q);
    size_t b = 3 * ch * sizeof(double) + 2 * sizeof(int) + 2 * sizeof(double) +
               IMFCS_NPARAM * sizeof(float) + sizeof(float) + 2 * sizeof(int) + 2 * sizeof(float);
    if (c.gls) b += (ch - 1) * (ch - 1) * sizeof(double);
    return b;
}

imfcs_config band_config(const imfcs_config &c, const BandGeom &g)
{
    imfcs_config b = c;
    b.height = g.in_rows;
    b.frames = c.num;
    b.first = 0;
    b.map_y0 = g.m;
    b.out_h = g.rows;
    return b;
}

}  // namespace

struct imfcs_bands {
    imfcs_config cfg;
    BandGeom g;
    imfcs_plan *pl = nullptr;
    size_t band_elems = 0;             // uint16 samples of one band buffer
    uint16_t *buf[2] = {};
    imfcs_outputs dout;
    bool dout_alloc = false;
    size_t bytes = 0;                  // device bytes held (plan, buffers, outputs)
    cudaStream_t copy = nullptr;
    cudaEvent_t copied[2] = {}, consumed[2] = {};
    std::vector<double> bg;            // per-pixel background image [height][width] (empty: scalar)
    ~imfcs_bands()
    {
        if (copy) cudaStreamSynchronize(copy);
        if (pl) imfcs_plan_destroy(pl);
        for (auto p : buf) if (p) cudaFree(p);
        void *o[] = {dout.acf, dout.var, dout.sd, dout.blocked_ind, dout.blocked_ok, dout.nb_mean, dout.nb_cov,
                     dout.fitres, dout.chi2, dout.fitted, dout.iterations, dout.bayes_prob, dout.covmats};
        for (auto p : o) if (p) cudaFree(p);
        for (int i = 0; i < 2; i++) {
            if (copied[i]) cudaEventDestroy(copied[i]);
            if (consumed[i]) cudaEventDestroy(consumed[i]);
        }
        if (copy) cudaStreamDestroy(copy);
    }
};

extern "C" int imfcs_band_window(const imfcs_config *cfg, int band_rows, int band, int *out_row0, int *new_row0,
                                 int *new_rows, int *in_row0, int *in_rows)
{
    std::string err;
    if (!config_valid(cfg, err)) { set_error(err); return -1; }
    if (band_rows <= 0) { set_error("band_rows must be positive"); return -1; }
    const BandGeom g = band_geom(*cfg, band_rows);
    if (band < 0 || band >= g.bands) { set_error("band index out of range"); return -1; }
    const BandWin w = band_win(*cfg, g, band);
    if (out_row0) *out_row0 = w.out_row0;
    if (new_row0) *new_row0 = w.new_row0;
    if (new_rows) *new_rows = w.new_rows;
    if (in_row0) *in_row0 = w.in_row0;
    if (in_rows) *in_rows = g.in_rows;
    return g.bands;
}

// Device bytes of a band job of `rows` output rows: the plan (scratch and
// tables), two band buffers, the band's outputs.  The trial plan binds no
// scratch, so sizing allocates only the plan's small tables.
static int bands_need(const imfcs_config &c, int rows, size_t *total)
{
    const BandGeom g = band_geom(c, rows);
    const imfcs_config bc = band_config(c, g);
    imfcs_plan *pl = nullptr;
    if (plan_create_ex(&bc, 0, bc.width, bc.height, false, &pl, true)) return 1;
    *total = plan_scratch_need(pl) + imfcs_plan_scratch_bytes(pl) +
             2 * (size_t)g.in_rows * c.width * c.num * sizeof(uint16_t) +
             (size_t)g.rows * c.out_w * output_bytes_per_pixel(c);
    imfcs_plan_destroy(pl);
    return 0;
}

extern "C" int imfcs_bands_create(const imfcs_config *cfg, int band_rows, size_t max_device_bytes,
                                  imfcs_bands **out)
{
    std::string err;
    if (!out) { set_error("null bands pointer"); return 1; }
    *out = nullptr;
    if (!config_valid(cfg, err)) { set_error(err); return 1; }
    const imfcs_config &c = *cfg;
    int rows = band_rows > 0 ? std::min(band_rows, c.out_h) : 0;
    if (rows == 0) {
        size_t budget = max_device_bytes;
        if (budget == 0) {
            size_t fr = 0, tot = 0;
            CK(cudaMemGetInfo(&fr, &tot));
            budget = fr / 10 * 9;
        }
        // the footprint is linear in the rows: measure it at one and two
        // rows, then shrink the estimate until it fits (alignment padding)
        size_t t1 = 0, t2 = 0, total = 0;
        if (bands_need(c, 1, &t1)) return 1;
        if (t1 > budget) { set_error("device budget below one band of one output row"); return 1; }
        if (c.out_h > 1 && bands_need(c, 2, &t2)) return 1;
        const size_t per_row = t2 > t1 ? t2 - t1 : t1;
        rows = (int)std::min<size_t>((size_t)c.out_h, 1 + (budget - t1) / per_row);
        while (rows > 1) {   // rows falls every pass: ends at one row at the latest
            if (bands_need(c, rows, &total)) return 1;
            if (total <= budget) break;
            rows = std::max(1, std::min(rows - 1, rows - rows / 16));
        }
    }
    const BandGeom g = band_geom(c, rows);
    const imfcs_config bc = band_config(c, g);
    imfcs_plan *pl = nullptr;
    if (imfcs_plan_create(&bc, &pl)) return 1;
    imfcs_bands *b = new imfcs_bands();
    b->cfg = c;
    b->g = g;
    b->pl = pl;
    b->band_elems = (size_t)g.in_rows * c.width * c.num;
    memset(&b->dout, 0, sizeof(b->dout));
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaMalloc(&b->buf[i], b->band_elems * sizeof(uint16_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->copy, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaEventCreateWithFlags(&b->copied[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->consumed[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        set_error(cuda_msg(e, "band buffers"));
        delete b;
        return 1;
    }
    b->bytes = imfcs_plan_scratch_bytes(pl) + 2 * b->band_elems * sizeof(uint16_t);
    *out = b;
    return 0;
}

extern "C" int imfcs_bands_destroy(imfcs_bands *b)
{
    delete b;
    return 0;
}

extern "C" int imfcs_bands_geometry(const imfcs_bands *b, int *band_rows, int *n_bands, size_t *device_bytes)
{
    if (!b) { set_error("null bands"); return 1; }
    if (band_rows) *band_rows = b->g.rows;
    if (n_bands) *n_bands = b->g.bands;
    if (device_bytes) *device_bytes = b->bytes;
    return 0;
}

extern "C" imfcs_plan *imfcs_bands_plan(imfcs_bands *b) { return b ? b->pl : nullptr; }

extern "C" int imfcs_bands_set_background_image(imfcs_bands *b, const double *host_bg)
{
    if (!b) { set_error("null bands"); return 1; }
    if (!host_bg) {
        b->bg.clear();
        return imfcs_plan_set_background_image(b->pl, nullptr);
    }
    const size_t n = (size_t)b->cfg.width * b->cfg.height;
    for (size_t i = 0; i < n; i++)
        if (!std::isfinite(host_bg[i]) || host_bg[i] < -2e9 || host_bg[i] > 2e9) {
            set_error("background image holds an invalid value");
            return 1;
        }
    b->bg.assign(host_bg, host_bg + n);
    return 0;
}

template <class T>
static cudaError_t band_d2h(T *host, const T *dev, size_t host_px, size_t dev_px, size_t n_px, size_t per_px,
                            cudaStream_t s)
{
    if (!host || !dev) return cudaSuccess;
    return cudaMemcpyAsync(host + host_px * per_px, dev + dev_px * per_px, n_px * per_px * sizeof(T),
                           cudaMemcpyDeviceToHost, s);
}

extern "C" int imfcs_bands_execute(imfcs_bands *b, const uint16_t *host_stack, const imfcs_outputs *host_out,
                                   void *stream)
{
    if (!b || !host_stack || !host_out) { set_error("null argument"); return 1; }
    // a background image set on the band plan directly would hold one
    // band's rows; imfcs_bands_set_background_image sets each band's
    if (b->bg.empty() && plan_job(b->pl).bg_trace) {
        set_error("set a per-pixel background image of bands with imfcs_bands_set_background_image");
        return 1;
    }
    const imfcs_config &c = b->cfg;
    const BandGeom &g = b->g;
    const cudaStream_t s = (cudaStream_t)stream;
    const size_t ch = (size_t)imfcs_chanum(c.p, c.q);
    const size_t bnp = (size_t)g.rows * c.out_w;
    if (!b->dout_alloc) {
        imfcs_outputs &d = b->dout;
        cudaError_t e = cudaSuccess;
        size_t add = 0;
#define OA(field, n)                                                                     \
    if (e == cudaSuccess && host_out->field) {                                           \
        const size_t nb = (size_t)(n) * sizeof(*d.field);                                \
        e = cudaMalloc((void **)&d.field, nb);                                           \
        if (e == cudaSuccess) add += nb;                                                 \
    }
        OA(acf, bnp * ch); OA(var, bnp * ch); OA(sd, bnp * ch);
        OA(blocked_ind, bnp); OA(blocked_ok, bnp); OA(nb_mean, bnp); OA(nb_cov, bnp);
        OA(fitres, bnp * IMFCS_NPARAM); OA(chi2, bnp); OA(fitted, bnp); OA(iterations, bnp);
        OA(bayes_prob, bnp * 2); OA(covmats, bnp * (ch - 1) * (ch - 1));
#undef OA
        if (e != cudaSuccess) { set_error(cuda_msg(e, "band output allocation")); return 1; }
        b->bytes += add;
        b->dout_alloc = true;
    }
    const size_t W = (size_t)c.width, H = (size_t)c.height;
    const size_t band_pitch = (size_t)g.in_rows * W * sizeof(uint16_t);
    // band k's rows of frames first..first+num-1 into buffer k & 1, after the
    // execution that last read that buffer
    auto enqueue_copy = [&](int k) -> int {
        const int i = k & 1;
        const BandWin w = band_win(c, g, k);
        if (w.in_row0 < 0 || w.in_row0 + g.in_rows > c.height) {
            set_error("band rows outside the image");
            return 1;
        }
        CK(cudaStreamWaitEvent(b->copy, b->consumed[i], 0));
        CK(cudaMemcpy2DAsync(b->buf[i], band_pitch, host_stack + ((size_t)c.first * H + w.in_row0) * W,
                             H * W * sizeof(uint16_t), band_pitch, c.num, cudaMemcpyHostToDevice, b->copy));
        CK(cudaEventRecord(b->copied[i], b->copy));
        return 0;
    };
    auto enqueue_all = [&]() -> int {
        if (enqueue_copy(0)) return 1;
        for (int k = 0; k < g.bands; k++) {
            const int i = k & 1;
            const BandWin w = band_win(c, g, k);
            // the next band's copy is queued before this band's results are read
            // back, so that it overlaps this band's execution
            if (k + 1 < g.bands && enqueue_copy(k + 1)) return 1;
            if (!b->bg.empty()) {
                // the band's rows of the background image; the previous band's
                // kernels read the plan's background sums until they finish
                CK(cudaStreamSynchronize(s));
                if (imfcs_plan_set_background_image(b->pl, b->bg.data() + (size_t)w.in_row0 * W)) return 1;
            }
            CK(cudaStreamWaitEvent(s, b->copied[i], 0));
            if (imfcs_plan_execute(b->pl, b->buf[i], &b->dout, s)) return 1;
            CK(cudaEventRecord(b->consumed[i], s));
            const imfcs_outputs &d = b->dout;
            const size_t hp = (size_t)w.new_row0 * c.out_w;                  // first new pixel, whole job
            const size_t dp = (size_t)(w.new_row0 - w.out_row0) * c.out_w;   // same pixel, in the band
            const size_t np = (size_t)w.new_rows * c.out_w;
            CK(band_d2h(host_out->acf, d.acf, hp, dp, np, ch, s));
            CK(band_d2h(host_out->var, d.var, hp, dp, np, ch, s));
            CK(band_d2h(host_out->sd, d.sd, hp, dp, np, ch, s));
            CK(band_d2h(host_out->blocked_ind, d.blocked_ind, hp, dp, np, 1, s));
            CK(band_d2h(host_out->blocked_ok, d.blocked_ok, hp, dp, np, 1, s));
            CK(band_d2h(host_out->nb_mean, d.nb_mean, hp, dp, np, 1, s));
            CK(band_d2h(host_out->nb_cov, d.nb_cov, hp, dp, np, 1, s));
            CK(band_d2h(host_out->fitres, d.fitres, hp, dp, np, IMFCS_NPARAM, s));
            CK(band_d2h(host_out->chi2, d.chi2, hp, dp, np, 1, s));
            CK(band_d2h(host_out->fitted, d.fitted, hp, dp, np, 1, s));
            CK(band_d2h(host_out->iterations, d.iterations, hp, dp, np, 1, s));
            CK(band_d2h(host_out->bayes_prob, d.bayes_prob, hp, dp, np, 2, s));
            CK(band_d2h(host_out->covmats, d.covmats, hp, dp, np, (ch - 1) * (ch - 1), s));
        }
        return 0;
    };
    if (enqueue_all()) {
        // copies already queued still read the caller's stack and write its
        // outputs: let them finish before the caller can free either
        cudaStreamSynchronize(b->copy);
        cudaStreamSynchronize(s);
        return 1;
    }
    return imfcs_plan_synchronize(b->pl, stream);
}
