// imfcs_ref_api.cu -- entry points with the reference's GpufitImFCS meaning
// (host buffers, synchronous), built on the same kernels as the whole-path API.
#include <math.h>
#include <stddef.h>
#include <string.h>

#include <string>
#include <vector>

#include "imfcs_args.h"
#include "imfcs_gb300.h"
#include "imfcs_host.h"

using namespace imfcs;

#define CKR(call)                                                            \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) { set_error(cuda_msg(_e, #call)); rc = 1; goto cleanup; } \
    } while (0)

namespace {

struct Scoped {
    std::vector<void *> ptrs;
    ~Scoped()
    {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T *&p, size_t n)
    {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
        if (e == cudaSuccess) { ptrs.push_back(q); p = (T *)q; }
        return e;
    }
};

size_t free_device_bytes()
{
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); return 0; }
    return fr;
}

}  // namespace

extern "C" int imfcs_reset_gpu(void)
{
    // No cudaDeviceReset on a shared device: finish outstanding work and
    // clear the error state of this thread.
    cudaError_t e = cudaDeviceSynchronize();
    cudaGetLastError();
    if (e != cudaSuccess) { set_error(cuda_msg(e, "cudaDeviceSynchronize")); return 1; }
    set_error("");
    return 0;
}

extern "C" int imfcs_is_binning_memory_sufficient(const imfcs_acf_parameters *p)
{
    if (!p) return 0;
    int frames = p->lastframe - p->firstframe + 1;
    double need = ((double)p->win_star * p->hin_star + (double)p->w_temp * p->h_temp) * frames * 4.0;
    return need < 0.9 * (double)free_device_bytes() ? 1 : 0;
}

extern "C" int imfcs_calc_binning(const float *in, float *out, const imfcs_acf_parameters *p)
{
    if (!in || !out || !p) { set_error("null argument"); return 1; }
    int rc = 0;
    Scoped m;
    const int frames = p->lastframe - p->firstframe + 1;
    const size_t nin = (size_t)p->win_star * p->hin_star * frames;
    const size_t nout = (size_t)p->w_temp * p->h_temp * frames;
    float *din = nullptr, *dout = nullptr;
    if (frames <= 0 || p->w_temp <= 0 || p->h_temp <= 0 ||
        p->w_temp + p->binningX - 1 > p->win_star || p->h_temp + p->binningY - 1 > p->hin_star) {
        set_error("invalid binning geometry");
        return 1;
    }
    CKR(m.alloc(din, nin));
    CKR(m.alloc(dout, nout));
    CKR(cudaMemcpy(din, in, nin * sizeof(float), cudaMemcpyHostToDevice));
    CKR(launch_binning(din, dout, p->win_star, p->hin_star, p->w_temp, p->h_temp, frames, p->binningX,
                       p->binningY, 0));
    CKR(cudaMemcpy(out, dout, nout * sizeof(float), cudaMemcpyDeviceToHost));
cleanup:
    return rc;
}

extern "C" int imfcs_calc_data_bleach_correction(const float *pixels, float *out,
                                                 const imfcs_acf_parameters *p)
{
    if (!pixels || !out || !p) { set_error("null argument"); return 1; }
    int rc = 0;
    Scoped m;
    const int frames = p->lastframe - p->firstframe + 1;
    const size_t nin = (size_t)p->w_temp * p->h_temp * frames;
    const size_t nout = (size_t)p->w_temp * p->h_temp * p->nopit;
    float *din = nullptr, *dout = nullptr;
    if (p->nopit <= 0 || p->ave <= 0 || (size_t)p->nopit * p->ave > (size_t)frames) {
        set_error("invalid nopit/ave");
        return 1;
    }
    CKR(m.alloc(din, nin));
    CKR(m.alloc(dout, nout));
    CKR(cudaMemcpy(din, pixels, nin * sizeof(float), cudaMemcpyHostToDevice));
    CKR(launch_bleach_average(din, dout, p->w_temp, p->h_temp, p->nopit, p->ave, 0));
    CKR(cudaMemcpy(out, dout, nout * sizeof(float), cudaMemcpyDeviceToHost));
cleanup:
    return rc;
}

static bool acf_config_from(const imfcs_acf_parameters *p, imfcs_config &c, std::string &err)
{
    memset(&c, 0, sizeof(c));
    const int frames = p->lastframe - p->firstframe + 1;
    if (frames <= 0) { err = "invalid frame range"; return false; }
    c.width = p->w_temp;
    c.height = p->h_temp;
    c.frames = frames;
    c.first = 0;
    c.num = frames;
    c.out_w = p->width;
    c.out_h = p->height;
    c.binx = c.biny = 1;          // the float stack is already binned
    c.pixbinx = p->pixbinX;
    c.pixbiny = p->pixbinY;
    c.cfx = p->cfXDistance;
    c.cfy = p->cfYDistance;
    c.background = 0;             // subtracted by the caller (java:14959-14983)
    c.p = (int)p->correlatorp;
    c.q = (int)p->correlatorq;
    c.frametime = p->frametime;
    c.bleach = p->bleachcorr_gpu ? IMFCS_BLEACH_POLYNOMIAL : IMFCS_BLEACH_NONE;
    c.poly_order = p->bleachcorr_gpu ? p->bleachcorr_order - 1 : 0;
    c.fitstart = 1;
    c.fitend = 0;
    if (p->cfXDistance < 0 || p->cfYDistance < 0) {
        err = "negative cross-correlation distances are not supported by calcACF (java:15296)";
        return false;
    }
    if (imfcs_chanum(c.p, c.q) != p->chanum) { err = "chanum does not match correlator P/Q"; return false; }
    return true;
}

extern "C" int imfcs_is_acf_memory_sufficient(const imfcs_acf_parameters *p)
{
    if (!p) return 0;
    const int frames = p->lastframe - p->firstframe + 1;
    const double npix = (double)p->width * p->height;
    const double ch = p->chanum;
    double need = (double)p->w_temp * p->h_temp * frames * 4.0        // input
                  + npix * ch * (8.0 * 3 + 16 + 20)                    // outputs, monitors, stats
                  + npix * 2 * 1000 * 4.0                              // averaged traces
                  + npix * 2 * ((frames + 255) / 256) * 8.0 * 12;      // segment scratch
    return need < 0.9 * (double)free_device_bytes() ? 1 : 0;
}

// Monomial coefficients in t (seconds) -> Legendre coefficients in
// u = t*uscale + uoff, by interpolation at order+1 Chebyshev nodes (FP64).
static void monomial_to_legendre(const double *c, int order, double uscale, double uoff, float *out)
{
    const int k = order + 1;
    std::vector<double> a(k * k), b(k);
    for (int i = 0; i < k; i++) {
        double u = cos(M_PI * (i + 0.5) / k);
        double t = (u - uoff) / uscale, f = 0.0, pw = 1.0;
        for (int q = 0; q < k; q++) { f += c[q] * pw; pw *= t; }
        b[i] = f;
        double l0 = 1.0, l1 = u;
        a[i * k + 0] = 1.0;
        if (k > 1) a[i * k + 1] = u;
        for (int n = 1; n + 1 < k; n++) {
            double l2 = ((2 * n + 1) * u * l1 - n * l0) / (n + 1);
            a[i * k + n + 1] = l2;
            l0 = l1;
            l1 = l2;
        }
    }
    for (int col = 0; col < k; col++) {   // Gaussian elimination with partial pivoting
        int pr = col;
        for (int r = col + 1; r < k; r++) if (fabs(a[r * k + col]) > fabs(a[pr * k + col])) pr = r;
        for (int q = 0; q < k; q++) std::swap(a[col * k + q], a[pr * k + q]);
        std::swap(b[col], b[pr]);
        for (int r = col + 1; r < k; r++) {
            double f = a[r * k + col] / a[col * k + col];
            for (int q = col; q < k; q++) a[r * k + q] -= f * a[col * k + q];
            b[r] -= f * b[col];
        }
    }
    std::vector<double> x(k);
    for (int i = k - 1; i >= 0; i--) {
        double s = b[i];
        for (int q = i + 1; q < k; q++) s -= a[i * k + q] * x[q];
        x[i] = s / a[i * k + i];
    }
    for (int i = 0; i < k; i++) out[i] = (float)x[i];
}

// Plan internals needed here (defined in imfcs_capi.cu).
namespace imfcs {
float *plan_bparams(imfcs_plan *pl);
const Job &plan_job(imfcs_plan *pl);
void plan_umap(imfcs_plan *pl, double &uscale, double &uoff);
const LagInfo &plan_laginfo(imfcs_plan *pl);
void plan_set_nb_only(imfcs_plan *pl, bool on);
}  // namespace imfcs

extern "C" int imfcs_calc_acf(const float *pixels, double *pixels1, double *blockvararray,
                              double *NBmean, double *NBcov, double *blocked1D,
                              const double *bleachcorr_params, double *samp, int *lag,
                              const imfcs_acf_parameters *p)
{
    if (!pixels || !p) { set_error("null argument"); return 1; }
    std::string err;
    imfcs_config c;
    if (!acf_config_from(p, c, err)) { set_error(err); return 1; }
    if (c.bleach == IMFCS_BLEACH_POLYNOMIAL && !bleachcorr_params) { set_error("bleach parameters missing"); return 1; }
    imfcs_plan *pl = nullptr;
    if (plan_create_ex(&c, 1, p->w_temp, p->h_temp, c.bleach == IMFCS_BLEACH_POLYNOMIAL, &pl)) return 1;
    int rc = 0;
    Scoped m;
    const Job &j = plan_job(pl);
    const int chanum = j.chanum, npix = j.npix;
    const size_t nin = (size_t)p->w_temp * p->h_temp * c.num;
    float *din = nullptr;
    double *acf = nullptr, *var = nullptr, *nbm = nullptr, *nbc = nullptr;
    int *bind = nullptr, *bok = nullptr;
    std::vector<double> h_acf, h_var;
    std::vector<int> h_ind, h_ok;
    imfcs_outputs o;
    memset(&o, 0, sizeof(o));
    CKR(m.alloc(din, nin));
    CKR(m.alloc(acf, (size_t)npix * chanum));
    CKR(m.alloc(var, (size_t)npix * chanum));
    CKR(m.alloc(nbm, npix));
    CKR(m.alloc(nbc, npix));
    CKR(m.alloc(bind, npix));
    CKR(m.alloc(bok, npix));
    CKR(cudaMemcpy(din, pixels, nin * sizeof(float), cudaMemcpyHostToDevice));
    if (c.bleach == IMFCS_BLEACH_POLYNOMIAL) {
        // caller's coefficients of the temp-grid pixel each trace starts at
        double us, uo;
        plan_umap(pl, us, uo);
        const int ncoef = p->bleachcorr_order;
        std::vector<float> bp((size_t)j.ntrace * kBleachStride, 0.f);
        for (int tr = 0; tr < j.ntrace; tr++) {
            int pix = tr < npix ? tr : tr - npix;
            int x0 = (pix % j.out_w) * j.pixbinx + (tr < npix ? 0 : j.cfx);
            int y0 = (pix / j.out_w) * j.pixbiny + (tr < npix ? 0 : j.cfy);
            const double *cc = bleachcorr_params + ((size_t)y0 * p->w_temp + x0) * ncoef;
            float *b = &bp[(size_t)tr * kBleachStride];
            monomial_to_legendre(cc, ncoef - 1, us, uo, b);
            b[9] = (float)cc[0];               // f0 = res[0] (java:9748)
            b[10] = (float)(1.0 / cc[0]);
            b[11] = 1.f;
            b[13] = (float)us;
            b[14] = (float)uo;
        }
        CKR(cudaMemcpy(plan_bparams(pl), bp.data(), bp.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    o.acf = acf; o.var = var; o.nb_mean = nbm; o.nb_cov = nbc; o.blocked_ind = bind; o.blocked_ok = bok;
    // N&B mode (agpufitjni.cu:5719-5720): lag 1 only; the ACF, variance and
    // blocking outputs are left as the caller passed them (the reference
    // copies back host arrays it never filled in this mode)
    plan_set_nb_only(pl, p->isNBcalculation != 0);
    if (plan_execute_any(pl, din, &o, nullptr)) { rc = 1; goto cleanup; }
    CKR(cudaDeviceSynchronize());
    if (p->isNBcalculation) {
        if (NBmean) CKR(cudaMemcpy(NBmean, nbm, npix * sizeof(double), cudaMemcpyDeviceToHost));
        if (NBcov) CKR(cudaMemcpy(NBcov, nbc, npix * sizeof(double), cudaMemcpyDeviceToHost));
        const LagInfo &li = plan_laginfo(pl);
        for (int x = 0; x < chanum; x++) {
            if (lag) lag[x] = li.lag[x];
            if (samp) samp[x] = (double)(1 << li.level[x]);
        }
        goto cleanup;
    }
    h_acf.resize((size_t)npix * chanum);
    h_var.resize((size_t)npix * chanum);
    h_ind.resize(npix);
    h_ok.resize(npix);
    CKR(cudaMemcpy(h_acf.data(), acf, h_acf.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(h_var.data(), var, h_var.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(h_ind.data(), bind, npix * sizeof(int), cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(h_ok.data(), bok, npix * sizeof(int), cudaMemcpyDeviceToHost));
    if (NBmean) CKR(cudaMemcpy(NBmean, nbm, npix * sizeof(double), cudaMemcpyDeviceToHost));
    if (NBcov) CKR(cudaMemcpy(NBcov, nbc, npix * sizeof(double), cudaMemcpyDeviceToHost));
    // lag-major outputs like the reference ([chanum][height][width])
    for (int x = 0; x < chanum; x++)
        for (int q = 0; q < npix; q++) {
            if (pixels1) pixels1[(size_t)x * npix + q] = h_acf[(size_t)q * chanum + x];
            if (blockvararray) blockvararray[(size_t)x * npix + q] = h_var[(size_t)q * chanum + x];
        }
    if (blocked1D)
        for (int q = 0; q < npix; q++) {
            blocked1D[q] = h_ind[q];
            blocked1D[npix + q] = h_ok[q];
        }
    {
        const LagInfo &li = plan_laginfo(pl);
        for (int x = 0; x < chanum; x++) {
            if (lag) lag[x] = li.lag[x];
            if (samp) samp[x] = (double)(1 << li.level[x]);
        }
    }
cleanup:
    imfcs_plan_destroy(pl);
    return rc;
}

// ---------------------------------------------------------------------------
// fit: Gpufit C API semantics (agpufitjni.cu:4332-4388, 4614-4640).
// ---------------------------------------------------------------------------
extern "C" int imfcs_fit(int n_fits, int n_points, const float *data, const float *weights,
                         int model_id, const float *initial_parameters, float tolerance,
                         int max_n_iterations, int num_valid_coefs, const int *parameters_to_fit,
                         int estimator_id, size_t user_info_size, const void *user_info,
                         float *output_parameters, int *output_states, float *output_chi_squares,
                         int *output_n_iterations)
{
    if (n_fits < 0 || n_points <= 0 || !data || !initial_parameters || !parameters_to_fit ||
        !output_parameters) {
        set_error("invalid argument");
        return -1;
    }
    if (estimator_id != 0) { set_error("only the LSE estimator is supported"); return -1; }
    if (model_id != IMFCS_MODEL_ACF_1D && model_id != IMFCS_MODEL_LINEAR_1D) {
        set_error("unsupported model id");
        return -1;
    }
    if (!user_info || user_info_size < (size_t)n_points * sizeof(float)) {
        set_error("user_info must hold n_points float abscissae");
        return -1;
    }
    if (n_fits == 0) return 0;
    const bool acf = model_id == IMFCS_MODEL_ACF_1D;
    const int nparam = acf ? IMFCS_ACF_1D_NPARAM : IMFCS_LINEAR_1D_NPARAM;
    const int np = acf ? IMFCS_NPARAM : num_valid_coefs;
    if (!acf && (num_valid_coefs < 1 || num_valid_coefs > IMFCS_LINEAR_1D_NPARAM)) {
        set_error("num_valid_coefs out of range");
        return -1;
    }
    int rc = 0;
    Scoped m;
    FitArgs a;
    memset(&a, 0, sizeof(a));
    a.nfits = n_fits;
    a.npts = n_points;
    a.model = model_id;
    a.np = np;
    for (int i = 0; i < np; i++)
        if (parameters_to_fit[i]) a.idx[a.k++] = i;
    a.max_iter = max_n_iterations > 0 ? max_n_iterations : 1;
    a.tol = tolerance > 0.f ? tolerance : 1e-30f;
    // host-side unit conversion (SI -> internal) and constants
    std::vector<float> init((size_t)n_fits * np), cst;
    for (int f = 0; f < n_fits; f++)
        for (int i = 0; i < np; i++)
            init[(size_t)f * np + i] = acf ? (float)(initial_parameters[(size_t)f * nparam + i] / param_unit(i))
                                           : initial_parameters[(size_t)f * nparam + i];
    if (acf) {
        cst.resize((size_t)n_fits * IMFCS_NCONST);
        for (int f = 0; f < n_fits; f++)
            for (int i = 0; i < IMFCS_NCONST; i++)
                cst[(size_t)f * IMFCS_NCONST + i] = initial_parameters[(size_t)f * nparam + IMFCS_NPARAM + i];
    }
    float *dy = nullptr, *dw = nullptr, *dx = nullptr, *dinit = nullptr, *dcst = nullptr, *dpar = nullptr,
          *dchi = nullptr;
    int *dst = nullptr, *dit = nullptr;
    std::vector<float> par;
    CKR(m.alloc(dy, (size_t)n_fits * n_points));
    if (weights) CKR(m.alloc(dw, (size_t)n_fits * n_points));
    CKR(m.alloc(dx, n_points));
    CKR(m.alloc(dinit, init.size()));
    if (acf) CKR(m.alloc(dcst, cst.size()));
    CKR(m.alloc(dpar, (size_t)n_fits * np));
    CKR(m.alloc(dchi, n_fits));
    CKR(m.alloc(dst, n_fits));
    CKR(m.alloc(dit, n_fits));
    CKR(cudaMemcpy(dy, data, sizeof(float) * n_fits * n_points, cudaMemcpyHostToDevice));
    if (weights) CKR(cudaMemcpy(dw, weights, sizeof(float) * n_fits * n_points, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(dx, user_info, sizeof(float) * n_points, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(dinit, init.data(), sizeof(float) * init.size(), cudaMemcpyHostToDevice));
    if (acf) CKR(cudaMemcpy(dcst, cst.data(), sizeof(float) * cst.size(), cudaMemcpyHostToDevice));
    a.y = dy;
    a.w = dw;
    a.x = dx;
    a.init = dinit;
    a.init_stride = np;
    a.cst = dcst;
    a.out_par = dpar;
    a.out_stride = np;
    a.out_chi2 = dchi;
    a.out_state = dst;
    a.out_iter = dit;
    {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        CKR(launch_lm(a, sms, 0));
    }
    CKR(cudaDeviceSynchronize());
    par.resize((size_t)n_fits * np);
    CKR(cudaMemcpy(par.data(), dpar, par.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (int f = 0; f < n_fits; f++) {
        for (int i = 0; i < nparam; i++) {
            float v;
            if (i < np) v = acf ? (float)(par[(size_t)f * np + i] * param_unit(i)) : par[(size_t)f * np + i];
            else v = initial_parameters[(size_t)f * nparam + i];
            output_parameters[(size_t)f * nparam + i] = v;
        }
    }
    if (output_states) CKR(cudaMemcpy(output_states, dst, sizeof(int) * n_fits, cudaMemcpyDeviceToHost));
    if (output_chi_squares) CKR(cudaMemcpy(output_chi_squares, dchi, sizeof(float) * n_fits, cudaMemcpyDeviceToHost));
    if (output_n_iterations) CKR(cudaMemcpy(output_n_iterations, dit, sizeof(int) * n_fits, cudaMemcpyDeviceToHost));
cleanup:
    return rc ? -1 : 0;
}
