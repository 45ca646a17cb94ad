/*
 * imfcs_gb300.h -- C ABI of the GB300-native imaging-FCS correlation-and-fit
 * engine (libimfcs_gb300.so).
 *
 * The library replaces the native side of the Imaging_FCS 1.52 plugin's GPU
 * path: the JNI binding GpufitImFCS.java (class gpufitImFCS.GpufitImFCS) over
 * libagpufit.so (agpufitjni.cu).  Every reference-facing entry point below
 * names the Java native method and the agpufitjni.cu implementation it
 * replaces.  Plain C types only: pointers, sizes and the two parameter
 * structs.  A JNI shim (jni/imfcs_jni.c in this repository) forwards the
 * Java natives to these functions.
 *
 * Conventions
 *  - Return value: 0 = success, nonzero = error; imfcs_get_last_error()
 *    returns the message of the last failure on the calling thread.
 *  - "host" pointers are ordinary host memory; "dev" pointers are CUDA device
 *    pointers of the current device; `stream` is a cudaStream_t (NULL = the
 *    legacy default stream).
 *  - No entry point resets the device (the reference ends each call with
 *    cudaDeviceReset, agpufitjni.cu:4781,4939,5769; on a shared GPU that is
 *    replaced by freeing this library's own allocations).
 *  - There is no CPU fallback: without a usable CUDA device every compute
 *    entry point fails with an error.
 */
#ifndef IMFCS_GB300_H
#define IMFCS_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define IMFCS_API __attribute__((visibility("default")))
#else
#define IMFCS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define IMFCS_NPARAM 11 /* N, D, vx, vy, G, F2, D2, F3, D3, Ftrip, Ttrip (SI units) */
#define IMFCS_NCONST 9  /* ax, ay, s, sz, rx, ry, fitobsvol, q2, q3 (SI units)      */

/* Bleach-correction modes (the plugin's cbBleachCor choices that reach the
 * correlator: "none", "Single Exp", "Double Exp", "Polynomial"). */
enum { IMFCS_BLEACH_NONE = 0, IMFCS_BLEACH_SINGLE_EXP = 1,
       IMFCS_BLEACH_DOUBLE_EXP = 2, IMFCS_BLEACH_POLYNOMIAL = 3 };

/* Fit states, identical to GpufitImFCS.FitState (GpufitImFCS.java:817-866). */
enum { IMFCS_STATE_CONVERGED = 0, IMFCS_STATE_MAX_ITERATIONS = 1,
       IMFCS_STATE_SINGULAR_HESSIAN = 2, IMFCS_STATE_NEG_CURVATURE_MLE = 3,
       IMFCS_STATE_GPU_NOT_READY = 4 };

/* Model ids, identical to GpufitImFCS.Model (GpufitImFCS.java:879-891). */
enum { IMFCS_MODEL_GAUSS_2D = 1, IMFCS_MODEL_ACF_1D = 2, IMFCS_MODEL_LINEAR_1D = 3 };
#define IMFCS_ACF_1D_NPARAM 20
#define IMFCS_LINEAR_1D_NPARAM 11

/* GpufitImFCS.ACFParameters (GpufitImFCS.java:453-486), field for field, in
 * the plugin's meaning.  Read by the reference at agpufitjni.cu:5462-5504. */
typedef struct imfcs_acf_parameters {
    int width, height;          /* output grid */
    int win_star, hin_star;     /* input width/height of the float stack */
    int w_temp, h_temp;         /* binned (stride-1 box sum) grid */
    int pixbinX, pixbinY;
    int binningX, binningY;
    int firstframe, lastframe;  /* 1-based, inclusive */
    int framediff;
    int cfXDistance, cfYDistance;
    double correlatorp, correlatorq;
    double frametime;
    int background;
    double mtab1, mtabchanumminus1, sampchanumminus1;
    int chanum;
    int isNBcalculation;
    int bleachcorr_gpu;
    int bleachcorr_order;       /* number of polynomial coefficients (order + 1) */
    int nopit, ave;
} imfcs_acf_parameters;

/* ------------------------------------------------------------------------ */
/* Device / status (reference-facing).                                       */
/* ------------------------------------------------------------------------ */

/* GpufitImFCS.isCudaAvailableInt (GpufitImFCS.java:389), agpufitjni.cu:4656.
 * Returns 1 when a CUDA device of compute capability 10.3 (GB300) is usable. */
IMFCS_API int imfcs_is_cuda_available(void);

/* GpufitImFCS.getCudaVersionAsArray (GpufitImFCS.java:403), agpufitjni.cu:4668.
 * Versions as major*1000 + minor*10. */
IMFCS_API int imfcs_get_cuda_version(int *runtime_version, int *driver_version);

/* GpufitImFCS.getLastError (GpufitImFCS.java:382), agpufitjni.cu:4643. */
IMFCS_API const char *imfcs_get_last_error(void);

/* GpufitImFCS.resetGPU (GpufitImFCS.java:491), agpufitjni.cu:4692.  Frees the
 * library's cached device buffers and plans; never resets the device. */
IMFCS_API int imfcs_reset_gpu(void);

/* ------------------------------------------------------------------------ */
/* Reference-facing compute entry points (host buffers, synchronous).        */
/* ------------------------------------------------------------------------ */

/* GpufitImFCS.isBinningMemorySufficient (GpufitImFCS.java:510),
 * agpufitjni.cu:4816-4853.  Returns 1 / 0. */
IMFCS_API int imfcs_is_binning_memory_sufficient(const imfcs_acf_parameters *p);

/* GpufitImFCS.calcBinning (GpufitImFCS.java:520), agpufitjni.cu:4860-4967:
 * stride-1 box sum of binningX x binningY over a float stack
 * in[t][hin_star][win_star] -> out[t][h_temp][w_temp], frames
 * firstframe..lastframe. */
IMFCS_API int imfcs_calc_binning(const float *in, float *out, const imfcs_acf_parameters *p);

/* GpufitImFCS.calcDataBleachCorrection (GpufitImFCS.java:501),
 * agpufitjni.cu:4708-4810: averages of `ave` frames, out[h][w][nopit], for
 * the pixels the correlator reads from pixels[t][h_temp][w_temp]. */
IMFCS_API int imfcs_calc_data_bleach_correction(const float *pixels, float *out,
                                      const imfcs_acf_parameters *p);

/* GpufitImFCS.isACFmemorySufficient (GpufitImFCS.java:531),
 * agpufitjni.cu:4974-5092.  Returns 1 / 0. */
IMFCS_API int imfcs_is_acf_memory_sufficient(const imfcs_acf_parameters *p);

/* GpufitImFCS.calcACF (GpufitImFCS.java:533), agpufitjni.cu:5364-5831.
 * pixels[t][h_temp][w_temp] (binned, background subtracted), outputs are
 * lag-major like the reference: pixels1[chanum][height][width] (ACF),
 * blockvararray[chanum][height][width], NBmean[height][width],
 * NBcov[height][width], blocked1D[2][height][width] (block index, success
 * flag).  bleachcorr_params[h_temp][w_temp][bleachcorr_order] are polynomial
 * coefficients in powers of t (seconds) when bleachcorr_gpu != 0.  samp and
 * lag receive the lag tables.  Semantics follow the plugin's Java CPU
 * correlator (java:9124-9648): time origin (x + 0.5) with 1-based x, the
 * averaged trace in int division, the zero-led lag-1 sequence of the
 * blocking transform. */
IMFCS_API int imfcs_calc_acf(const float *pixels, double *pixels1, double *blockvararray,
                   double *NBmean, double *NBcov, double *blocked1D,
                   const double *bleachcorr_params, double *samp, int *lag,
                   const imfcs_acf_parameters *p);

/* GpufitImFCS.fit (GpufitImFCS.java:323), agpufitjni.cu:4614-4640 and the
 * Gpufit C API gpufit() (agpufitjni.cu:4332-4388).  Models ACF_1D (20
 * parameters: the 11 FCS parameters then ax, ay, s, sz, rx, ry, fitobsvol,
 * q2, q3; user_info = n_points float lag times) and LINEAR_1D (polynomial with
 * num_valid_coefs coefficients; user_info = n_points float abscissae).
 * Estimator 0 (LSE) only.  Outputs per fit: parameters, state, chi-square
 * (sum of weighted squared residuals) and iteration count. */
IMFCS_API int imfcs_fit(int n_fits, int n_points, const float *data, const float *weights,
              int model_id, const float *initial_parameters, float tolerance,
              int max_n_iterations, int num_valid_coefs, const int *parameters_to_fit,
              int estimator_id, size_t user_info_size, const void *user_info,
              float *output_parameters, int *output_states, float *output_chi_squares,
              int *output_n_iterations);

/* No counterpart in the reference.  The same fit as imfcs_fit on DEVICE
 * buffers, asynchronous on `stream`, and without any device allocation: for
 * callers that cannot allocate at fit time -- a host pipeline that keeps other
 * streams busy (cudaMalloc/cudaFree synchronise the device and would stall
 * them), or one whose device memory is fully reserved by its own pool.
 * data/weights [n_fits][n_points], initial_parameters and output_parameters
 * [n_fits][20 (ACF_1D) or 11 (LINEAR_1D)], user_info = n_points float
 * abscissae, outputs (states, chi-squares, iterations: each nullable) are
 * device pointers; parameters_to_fit is a host array.  Scratch is a fixed
 * file-scope device array sized for IMFCS_FIT_NOALLOC_MAX_FITS fits (2 MB);
 * larger batches are rejected with an error (split them).  No part of the
 * scratch needs to start at zero: each call writes every element it reads.
 * Every call looks up the scratch address in the current context
 * (cudaGetSymbolAddress, which allocates nothing), so the entry point stays
 * valid after a cudaDeviceReset or in another context.  Calls that
 * overlap on one device (other host threads or streams) share the scratch
 * and race: serialise them.  Returns 0 / -1 (imfcs_get_last_error). */
#define IMFCS_FIT_NOALLOC_MAX_FITS 16384
IMFCS_API int imfcs_fit_device_noalloc(int n_fits, int n_points, const float *data, const float *weights,
              int model_id, const float *initial_parameters, float tolerance,
              int max_n_iterations, int num_valid_coefs, const int *parameters_to_fit,
              const float *user_info, float *output_parameters, int *output_states,
              float *output_chi_squares, int *output_n_iterations, void *stream);

/* ------------------------------------------------------------------------ */
/* GB300-native whole-path API (uint16 stack -> ACF, variance, fits).        */
/* ------------------------------------------------------------------------ */

/* One correlation job over a raw uint16 stack [frames][height][width]:
 * output pixel (ox, oy) correlates the binx x biny window at raw
 * ((map_x0+ox)*pixbinx, (map_y0+oy)*pixbiny) with the window displaced by
 * (cfx, cfy) (the correlateROI CPU loop, java:8457-8556). */
typedef struct imfcs_config {
    int width, height, frames;   /* raw stack geometry */
    int first, num;              /* 0-based first frame, number of frames */
    int out_w, out_h, map_x0, map_y0;
    int binx, biny, pixbinx, pixbiny;
    int cfx, cfy;
    int background;              /* counts per raw pixel (java getIntensity) */
    int p, q;                    /* correlator: P = 16, Q >= 1 (chanum = P+(Q-1)P/2+1) */
    double frametime;            /* seconds */
    int bleach, poly_order;      /* IMFCS_BLEACH_*, polynomial order 1..8 */
    int gls, bayes, do_fit;      /* GLS covariance/fit, Bayes 1-vs-2, fit at all */
    int fitstart, fitend;        /* OLS fit range (lag indices), java:10358-10369 */
    int max_iter;                /* LM iteration cap (java:199: 2000) */
    double init[IMFCS_NPARAM];   /* initial values (SI) */
    int free_mask[IMFCS_NPARAM]; /* 1 = fitted, 0 = held at init */
    double cst[IMFCS_NCONST];    /* model constants (SI) */
} imfcs_config;

/* Output buffers of a job ([pixel][...] with pixel = oy*out_w + ox).
 * Any pointer may be NULL to skip that output. */
typedef struct imfcs_outputs {
    double *acf;         /* [npix][chanum]  (GLS: mcov, as java:9638-9642)    */
    double *var;         /* [npix][chanum]  blocked variance                 */
    double *sd;          /* [npix][chanum]                                   */
    int *blocked_ind;    /* [npix] blocking index                            */
    int *blocked_ok;     /* [npix] blockIndS                                 */
    double *nb_mean;     /* [npix] lag-1 direct monitor (N&B)                */
    double *nb_cov;      /* [npix] lag-1 covariance (N&B)                    */
    float *fitres;       /* [npix][11] fitted parameters (SI), NaN if failed */
    float *chi2;         /* [npix] reduced chi-square as java:10403-10406    */
    int *fitted;         /* [npix] 1 if the fit succeeded                    */
    int *iterations;     /* [npix] LM iterations                             */
    float *bayes_prob;   /* [npix][2] model probabilities (1 and 2 comp.)    */
    double *covmats;     /* [npix][(chanum-1)^2] regularised covariance (GLS) */
} imfcs_outputs;

/* Number of correlation channels for (p, q): p + (q-1)*p/2 + 1. */
IMFCS_API int imfcs_chanum(int p, int q);

/* Plans hold the device scratch of one configuration; create once, execute
 * many times.  Not thread-safe per plan. */
typedef struct imfcs_plan imfcs_plan;
IMFCS_API int imfcs_plan_create(const imfcs_config *cfg, imfcs_plan **plan);
IMFCS_API int imfcs_plan_destroy(imfcs_plan *plan);
/* Bytes of device scratch the plan holds. */
IMFCS_API size_t imfcs_plan_scratch_bytes(const imfcs_plan *plan);

/* Diagnostic (no counterpart in the reference): copies the per-trace bleach
 * parameters of the last execution to host memory, 16 floats per trace
 * ([0..8] polynomial coefficients, or A, tau, C / A1, tau1, A2, tau2, C of
 * the exponential fit; [9] f0, [11] valid flag, [12] centre).  Returns the
 * number of traces. */
IMFCS_API int imfcs_plan_bleach_params(const imfcs_plan *plan, float *host_out, int max_traces);

/* Diagnostic (no counterpart in the reference): number of CUDA kernels the
 * last imfcs_plan_execute / imfcs_plan_execute_host launched. */
IMFCS_API int imfcs_plan_kernel_launches(const imfcs_plan *plan);

/* Stage timing (no counterpart in the reference): when enabled, every
 * execution records CUDA events around its stages on the execution stream;
 * imfcs_plan_stage_times() (after the stream is synchronised) returns the
 * durations in ms of the last execution: [0] averaged trace + bleach fit,
 * [1] the streaming pass over the raw stack (corrected level-0 stream and
 * the lags' monitors), [2] blocking transform, [3] correlator (level pairs,
 * top levels, G and variance), [4] GLS covariance, [5] fits.  Returns the
 * number of stages written. */
IMFCS_API int imfcs_plan_set_timing(imfcs_plan *plan, int enable);
IMFCS_API int imfcs_plan_stage_times(const imfcs_plan *plan, float *ms, int max_stages);

/* Correlator tile of the level chain (no counterpart in the reference, whose
 * kernels use fixed 16x16 thread blocks, agpufitjni.cu:5521-5531): `cta`
 * output pixels per CTA (32 or 64), the pair kernels' frame segments
 * 2^seg_extra (0..2) and the tail kernel's 2^tail_extra (0..4) times the
 * shortest legal segment (the block length of the blocked variance).
 * Results agree to FP32 rounding of the per-segment sums. */
typedef struct imfcs_corr_tile {
    int cta;
    int seg_extra;
    int tail_extra;
    float ms;                 /* median correlator time of the trial */
} imfcs_corr_tile;
IMFCS_API int imfcs_plan_set_corr_tile(imfcs_plan *plan, int cta, int seg_extra, int tail_extra);
IMFCS_API int imfcs_plan_get_corr_tile(const imfcs_plan *plan, int *cta, int *seg_extra, int *tail_extra);
/* Autotuner: executes the plan once on dev_stack (outputs as
 * imfcs_plan_execute), then times the correlator (median of three launches
 * after one warm-up) at the six (cta, seg_extra) tiles with the tail
 * segment alike, then at the other tail segments of the fastest, and keeps
 * the fastest (10 trials).  Writes up to max_trials trials.  Synchronises
 * `stream`. */
IMFCS_API int imfcs_plan_autotune(imfcs_plan *plan, const uint16_t *dev_stack, const imfcs_outputs *dev_out,
                        void *stream, imfcs_corr_tile *trials, int max_trials, int *n_trials);

/* Stack ingest (replaces the plugin's ImageJ read, getVoxels
 * Imaging_FCS_1_52.java:14791 and GPU_get_pixels 14913-14983, which copy
 * every frame into a Java float array): uncompressed 16-bit single-channel
 * TIFF stacks in either byte order, one IFD per frame (any strips) or
 * ImageJ's single-IFD stacks ("images=N" in the description, frames
 * contiguous).  Frames come out as uint16 [t][height][width] in native
 * byte order.  imfcs_tiff_read_device copies through two pinned 64 MB
 * staging buffers used in turn (the file read of a chunk overlaps the
 * previous chunk's copy) and orders `stream` after the copies. */
typedef struct imfcs_tiff imfcs_tiff;
IMFCS_API int imfcs_tiff_open(const char *path, imfcs_tiff **tiff, int *width, int *height, int *frames);
IMFCS_API int imfcs_tiff_read(imfcs_tiff *tiff, int first, int count, uint16_t *host_out);
IMFCS_API int imfcs_tiff_read_device(imfcs_tiff *tiff, int first, int count, uint16_t *dev_out, void *stream);
IMFCS_API int imfcs_tiff_close(imfcs_tiff *tiff);

/* Background-file statistics (loadBGRFile, Imaging_FCS_1_52.java:6988-7103)
 * of a device-resident background stack dev_stack[frames][height][width]:
 * per-pixel mean and variance over all frames, lag-1 covariance (means of
 * frames 1..f-1 and 2..f), row means [height] and column means [width];
 * device outputs, any may be NULL; identical to the Java's doubles.  The
 * mean image feeds imfcs_plan_set_background_image.  Asynchronous. */
IMFCS_API int imfcs_background_stats(const uint16_t *dev_stack, int width, int height, int frames, double *mean,
                           double *var, double *covar, double *row_mean, double *col_mean, void *stream);

/* Batches (no counterpart in the reference, which repeats one JNI call per
 * binning, Imaging_FCS_1_52.java:11146-11166): several jobs -- binnings,
 * cross-correlation offsets, ROIs of different sizes -- over one stack
 * (every config has the same width, height, frames, first and num), run as
 * one CUDA graph.  Jobs are spread over `lanes` concurrent branches of the
 * graph; jobs of one lane run one after another on one scratch arena sized
 * for the largest of them.  The graph is captured at the first execution
 * and again whenever the stack, the outputs, the lanes or a tile change. */
typedef struct imfcs_batch imfcs_batch;
IMFCS_API int imfcs_batch_create(const imfcs_config *jobs, int n_jobs, int lanes, imfcs_batch **batch);
IMFCS_API int imfcs_batch_destroy(imfcs_batch *batch);
/* outs: n_jobs device output sets (as imfcs_plan_execute).  Asynchronous. */
IMFCS_API int imfcs_batch_execute(imfcs_batch *batch, const uint16_t *dev_stack, const imfcs_outputs *outs,
                        void *stream);
/* Waits for `stream` and reports device-side errors of every job. */
IMFCS_API int imfcs_batch_synchronize(imfcs_batch *batch, void *stream);
/* Autotuner: tunes every job's correlator tile (imfcs_plan_autotune), times
 * each job alone, then for 1..max_lanes lanes assigns jobs to lanes by
 * longest measured time first and times the whole graph (best of two after
 * one warm-up);
 * keeps the fastest lane count.  lane_ms[l-1] receives the time with l lanes
 * (max_lanes entries, 0 where the arenas did not fit in device memory).
 * Synchronises `stream`. */
IMFCS_API int imfcs_batch_autotune(imfcs_batch *batch, const uint16_t *dev_stack, const imfcs_outputs *outs,
                         void *stream, int max_lanes, float *lane_ms);
/* Per job: output pixels, channels, lane, correlator tile and measured time
 * (ms, 0 before autotuning). */
IMFCS_API int imfcs_batch_job_info(const imfcs_batch *batch, int job, int *npix, int *chanum, int *lane,
                         int *cta, int *seg_extra, int *tail_extra, float *ms);
IMFCS_API int imfcs_batch_lanes(const imfcs_batch *batch);
/* Device bytes of the scratch arenas and of the jobs' own tables. */
IMFCS_API size_t imfcs_batch_scratch_bytes(const imfcs_batch *batch);
/* Kernels the graph launches per execution. */
IMFCS_API int imfcs_batch_kernel_launches(const imfcs_batch *batch);

/* Runs the whole path on a device-resident stack; outputs are device
 * pointers.  Asynchronous on `stream`. */
IMFCS_API int imfcs_plan_execute(imfcs_plan *plan, const uint16_t *dev_stack, const imfcs_outputs *dev_out,
                       void *stream);

/* Same path with host buffers: copies the stack (host, ideally pinned) in,
 * runs, copies the outputs back and synchronises. */
IMFCS_API int imfcs_plan_execute_host(imfcs_plan *plan, const uint16_t *host_stack,
                            const imfcs_outputs *host_out, void *stream);

/* Asynchronous form of imfcs_plan_execute_host for a sequence of stacks:
 * enqueues the stack copy (on the plan's own copy stream, into one of two
 * device stack buffers used in turn), the execution and the copies of the
 * results on `stream`, and returns at once.  The copy of the next stack
 * then overlaps the current execution.  With page-locked (pinned) host
 * buffers the host thread does not wait; the host stack must stay unchanged
 * until the execution that reads it has completed and the outputs are valid
 * only after imfcs_plan_synchronize.  Successive calls on one plan write the
 * same host output buffers unless the caller passes different ones. */
IMFCS_API int imfcs_plan_execute_host_async(imfcs_plan *plan, const uint16_t *host_stack,
                                  const imfcs_outputs *host_out, void *stream);
/* Waits for the plan's executions on `stream`; reports a device-side error. */
IMFCS_API int imfcs_plan_synchronize(imfcs_plan *plan, void *stream);

/* Band-streamed execution of a host stack larger than the device memory the
 * caller grants (no counterpart in the reference: the plugin copies the
 * whole stack to the device as one float array, Imaging_FCS_1_52.java:
 * 14908-14983, agpufitjni.cu:5510,5586).  The job's output rows are split
 * into bands of band_rows rows (0: the most rows whose device footprint --
 * plan scratch, two band buffers, outputs -- fits in max_device_bytes; 0
 * bytes: 90 % of the free device memory).  Each band's input rows (its
 * windows plus the (binning-1) + |cfy| rows of halo) of frames first ..
 * first+num-1 go to the device in one 2D copy on an internal copy stream
 * while the previous band computes; results equal imfcs_plan_execute_host's
 * on the whole stack, since output pixels are independent.
 * imfcs_bands_execute returns after the results are in host_out (pinned
 * host buffers let copies and computation overlap). */
typedef struct imfcs_bands imfcs_bands;
IMFCS_API int imfcs_bands_create(const imfcs_config *cfg, int band_rows, size_t max_device_bytes,
                                 imfcs_bands **bands);
IMFCS_API int imfcs_bands_destroy(imfcs_bands *bands);
/* Output rows per band, number of bands, device bytes held. */
IMFCS_API int imfcs_bands_geometry(const imfcs_bands *bands, int *band_rows, int *n_bands, size_t *device_bytes);
/* The plan that runs every band (for its tile, timing and surrogate settings;
 * a background image goes through imfcs_bands_set_background_image). */
IMFCS_API imfcs_plan *imfcs_bands_plan(imfcs_bands *bands);
/* Per-pixel background image [height][width] of the whole input frame (as
 * imfcs_plan_set_background_image; NULL: the scalar background); each band
 * takes its rows (copied: the caller's array may be freed). */
IMFCS_API int imfcs_bands_set_background_image(imfcs_bands *bands, const double *host_bg);
IMFCS_API int imfcs_bands_execute(imfcs_bands *bands, const uint16_t *host_stack, const imfcs_outputs *host_out,
                                  void *stream);
/* FP32 issue-rate probe (no counterpart in the reference): FMA
 * instructions per second the device sustains over independent chains on
 * every SM (best of five timed launches); the denominator of the fit
 * stage's roofline. */
IMFCS_API int imfcs_measure_fp32_fma_rate(double *fma_per_s, void *stream);

/* Band split without a device (host arithmetic only): band `band` of a job
 * split into bands of band_rows output rows -- the first output row it
 * computes, the first and the number of output rows it adds (the last band
 * is moved up to end at the job's last row), the input row of its buffer's
 * first row and its input rows.  Returns the number of bands, -1 on an invalid argument. */
IMFCS_API int imfcs_band_window(const imfcs_config *cfg, int band_rows, int band, int *out_row0, int *new_row0,
                                int *new_rows, int *in_row0, int *in_rows);

/* FCS diffusion law (dlfit, java:11007-11231, determineDiffusionLaw 8190-8250,
 * fitDiffLaw 8253-8295): for binnings 1..n_bin the whole path is run on the
 * device-resident stack; out[3*n_bin] = {Aeff [um^2], mean D [um^2/s],
 * variance of D} per binning, line[2] = intercept, slope of Aeff/D vs Aeff
 * fitted over binnings fit_lo..fit_hi (1-based).  `cfg` supplies everything
 * except the binning and output grid, which follow the "All", non-overlap
 * mode of the plugin. */
IMFCS_API int imfcs_diffusion_law(const imfcs_config *cfg, const uint16_t *dev_stack, int n_bin,
                        int fit_lo, int fit_hi, double pixel_size_m, double psf_m,
                        double *out, double *line, void *stream);

/* PSF calibration (determinePSF, java:8115-8160): for psf_count < 10 PSF
 * sizes psf_m[i] (1/e^2 radius, m) and binnings 1..n_bin (the "All",
 * non-overlap mode of dlfit), out[i][3][n_bin] receives what the plugin
 * tabulates per binning: the label u + bin_start of binning u + 1, the mean
 * fitted D [um^2/s] and the variance of D divided by
 * sqrt(width / (u + 1) * height / (u + 1)) (Java int arithmetic).  The
 * correlations are computed once per binning and fitted for every PSF.
 * At least 20 x 20 pixels are required, as in the plugin. */
IMFCS_API int imfcs_psf_calibration(const imfcs_config *cfg, const uint16_t *dev_stack, int n_bin, int bin_start,
                          const double *psf_m, int psf_count, double pixel_size_m, double *out,
                          void *stream);

/* Seeded 2D Brownian-motion stack simulator (semantics of simulateACF2D,
 * java:13854-14409: Brownian steps, Gaussian PSF photon scatter, Poisson
 * emission, camera offset).  Writes dev_stack[frames][height][width].
 * d_tile_map (optional, [ceil(h/16)][ceil(w/16)] um^2/s) gives D per 16x16
 * pixel tile; fraction2/d2 add a second species; tau_bleach (s, 0 = none)
 * bleaches the emission exponentially. */
typedef struct imfcs_sim_params {
    int width, height, frames;
    double frametime;            /* s */
    int steps_per_frame;
    double pixel_size;           /* um, object space */
    double psf_radius;           /* 1/e^2 radius, um */
    double density;              /* particles per um^2 */
    double d1, d2, fraction2;    /* um^2/s */
    double cps;                  /* photons per second per particle */
    double tau_bleach;           /* s */
    int offset;                  /* camera offset, counts */
    double read_noise;           /* Gaussian read noise sigma, counts */
    double margin;               /* um around the detector */
    uint64_t seed;
} imfcs_sim_params;
IMFCS_API int imfcs_simulate(const imfcs_sim_params *sp, const float *dev_d_tile_map, uint16_t *dev_stack,
                   void *stream);

/* ------------------------------------------------------------------------
 * Learned fit seeds.  No counterpart in the reference, whose fits all start
 * from the configured initial values (java:1958-1970, passed to the GPU fit
 * at java:15112-15185).  A small MLP (128 -> 256 -> 256 -> 4, GELU, BF16
 * tensor-core kernels with FP32 accumulation and FP32 master weights) maps
 * a pixel's normalised ACF and its standard deviation, lags 1..64, to
 * standardised predictions of log D [um^2/s], log(N G(1)), G_inf / G(1) and
 * the fraction of a second component; a plan with a surrogate attached
 * starts each pixel's LM fit from those predictions and refits from the
 * configured initial values where the seeded fit fails (see
 * imfcs_plan_set_surrogate).
 * ---------------------------------------------------------------------- */
typedef struct imfcs_surrogate imfcs_surrogate;
#define IMFCS_SURROGATE_INPUTS 128
#define IMFCS_SURROGATE_OUTPUTS 4
/* Parameter count: W1[128][256] b1[256] W2[256][256] b2[256] W3[256][4] b3[4]
 * (row-major, x W + b); the host parameter arrays of get/set_params hold
 * these followed by the 4 target means and the 4 target standard deviations. */
IMFCS_API size_t imfcs_surrogate_param_count(void);
IMFCS_API int imfcs_surrogate_create(uint64_t seed, imfcs_surrogate **out);
IMFCS_API int imfcs_surrogate_destroy(imfcs_surrogate *s);
IMFCS_API int imfcs_surrogate_get_params(const imfcs_surrogate *s, float *host_params);
IMFCS_API int imfcs_surrogate_set_params(imfcs_surrogate *s, const float *host_params);
/* Inputs from correlator outputs (dev acf/var [npix][chanum], chanum >= 65):
 * dev_x[npix][128] = G(i)/G(1) for i = 1..64, then sd(i)/|G(1)|. */
IMFCS_API int imfcs_surrogate_features(int npix, int chanum, const double *dev_acf, const double *dev_var,
                                       float *dev_x, void *stream);
/* One forward + backward pass of the mean squared error against standardised
 * targets ((t - mean) / std with the handle's current mean and std) over n
 * samples: host_grads[param_count] (nullable) and *loss (nullable). */
IMFCS_API int imfcs_surrogate_gradients(imfcs_surrogate *s, const float *dev_x, const float *dev_t, int n,
                                        float *host_grads, double *loss);
/* Adam training: sets the target standardisation from dev_t [n][4], then
 * `steps` minibatch steps of `batch` consecutive samples at seeded random
 * offsets (shuffle the samples beforehand).  loss_history[steps] nullable. */
IMFCS_API int imfcs_surrogate_train(imfcs_surrogate *s, const float *dev_x, const float *dev_t, int n, int steps,
                                    int batch, float learning_rate, uint64_t seed, float *loss_history,
                                    void *stream);
/* De-standardised predictions dev_out[n][4]. */
IMFCS_API int imfcs_surrogate_predict(imfcs_surrogate *s, const float *dev_x, int n, float *dev_out, void *stream);

/* Attaches a surrogate to a plan's do_fit LM (NULL or mode 0 detaches).
 * mode 1: seeded LM, then LM from the configured initial values for every
 *         pixel whose seeded fit did not converge or ended with N <= 0,
 *         D <= 0 or a non-finite parameter;
 * mode 2: as mode 1, and plain LM from the configured initial values also
 *         runs for every pixel; a pixel whose seeded chi^2 exceeds the plain
 *         chi^2 by more than 1 % takes the plain result (the plain fit is the
 *         arbiter of the seeded one).
 * The plan keeps the pointer; the surrogate must outlive its use. */
IMFCS_API int imfcs_plan_set_surrogate(imfcs_plan *plan, imfcs_surrogate *s, int mode);
/* Per-pixel background image, the plugin's background-file mode (bgrloaded:
 * getIntensity java:9671-9673, calcIntensityTrace java:9842-9845).
 * host_bg[height][width] in the input frame's geometry holds each raw
 * pixel's mean background; its value rounded as Math.round does replaces the
 * scalar background of that pixel.  As in the reference, the averaged
 * intensity traces (the bleach fits' input) of a cross-correlation's second
 * window subtract the background of the first window's pixels.  NULL
 * restores the scalar background.  uint16 plans only (the float-stack
 * calcACF path receives background-subtracted data, java:14959-14983). */
IMFCS_API int imfcs_plan_set_background_image(imfcs_plan *plan, const double *host_bg);

/* After an execute with a surrogate attached (synchronise first): pixels
 * refit from the configured initial values, and (mode 2) pixels whose
 * seeded chi^2 exceeded the plain chi^2 by more than 1 %. */
IMFCS_API int imfcs_plan_surrogate_stats(const imfcs_plan *plan, int *n_refit, int *n_worse);

#ifdef __cplusplus
}
#endif
#endif
