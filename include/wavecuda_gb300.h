/*
 * wavecuda_gb300 -- C ABI of the GB300 (sm_103a) wavelet library.
 *
 * Two layers:
 *
 *  1. The reference's own R-facing symbols, same names and signatures as
 *     rfunctions.cuh:17-36 of the reference, so that the R package's
 *     useDynLib(wavecuda, ...) bindings (NAMESPACE:26-30) resolve against this
 *     library unchanged.  Every computation runs on the GPU: the Rcpu* symbols
 *     are served by the same device path as the Rgpu* ones.
 *
 *  2. Status-returning entry points (wc_*): host-buffer calls, device-pointer
 *     calls on a caller stream, batched smoothing, adjoints and small runtime
 *     helpers.  Every wc_* call returns WC_OK (0) or an error code and never
 *     exits the process; wc_last_error() describes the last failure.
 *
 * Codes (wvtheads.h:14-38, rfunctions.cuh:13-15 of the reference):
 *   sense     FWD 1, BWD 0
 *   filter    HAAR 1, D4 2, C6 3, LA8 4          (filterlen 2, 4, 6, 8)
 *   ttype     DWT 0, MODWT (time ordered) 1, MODWT (packet ordered) 2
 *   hardness  HARD 0, SOFT 1
 *   threshtype MANUAL 0, UNIV 1, CV 2
 *   levels are 0-based in C (R's min.level - 1).
 *
 * Layouts (haar.cpp:9-30, haar.cpp:561-585):
 *   DWT   x (len values), transformed in place, interleaved: after J levels the
 *         level-l details (1-based) sit at indices = 2^(l-1) mod 2^l and the
 *         level-J scaling coefficients at indices = 0 mod 2^J.
 *   MODWT xmod = [s_1 | d_1 | s_2 | d_2 | ... | s_J | d_J], 2*len*J values.
 *   MODWT packet ordered (haar.cpp:305-398, daub4.cpp:392-484): level block
 *         l (2*len values) holds 2^(l+1) packets; packet sh has the (s, d)
 *         pairs of time positions rev(sh, l+1) + 2^(l+1) k, interleaved
 *         (convert_modwt_level, wavutils.cpp:569-600).  The transform, host
 *         thresholding and smoothing calls accept it; the batched, tuning and
 *         device-pointer MODWT calls take time order.
 *
 * Precision codes (wc_* calls; the R symbols use the process default):
 *   WC_F64_EXACT  FP64, every product and sum rounded in the reference's order
 *                 (no FMA contraction): results bit-identical to the
 *                 reference CPU path.
 *   WC_F64_FAST   FP64 data in HBM, arithmetic in double-float on the FP32
 *                 pipes (about 2^-48 relative per operation).
 *   WC_F32        FP32 data and arithmetic.
 */
#ifndef WAVECUDA_GB300_H
#define WAVECUDA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define WC_API __attribute__((visibility("default")))
#else
#define WC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------- status codes */
#define WC_OK 0
#define WC_ERR_ARG 1         /* invalid argument (length, code, pointer) */
#define WC_ERR_LEVELS 2      /* level count or level range rejected */
#define WC_ERR_CUDA 3        /* a CUDA runtime call failed */
#define WC_ERR_NOMEM 4       /* device or pinned host allocation failed */
#define WC_ERR_UNSUPPORTED 5 /* combination not provided */
#define WC_ERR_NODEVICE 6    /* no usable CUDA device */
#define WC_ERR_TIMEOUT 7     /* a bounded device-side wait gave up; results incomplete */

#define WC_F64_EXACT 0
#define WC_F64_FAST 1
#define WC_F32 2

/* ------------------------------------------------- 1. reference symbols */

/* rfunctions.cu:3 (RcpuTransform).  FWD DWT: x in place.  FWD MODWT: reads x,
 * writes the first 2*len*J values of xmod.  BWD DWT: x in place.  BWD MODWT:
 * reads xmod, writes x.  nlevels 0 means the maximum.  Errors are printed. */
WC_API void RcpuTransform(double* x, double* xmod, int* len, int* sense, int* nlevels,
                   int* ttype, int* filter, int* filterlen);

/* rfunctions.cu:21 (RgpuTransform).  Same contract as RcpuTransform. */
WC_API void RgpuTransform(double* x, double* xmod, int* len, int* sense, int* nlevels,
                   int* ttype, int* filter, int* filterlen);

/* rfunctions.cu:59 (RcpuThreshold).  Thresholds x (DWT) or xmod (MODWT) in
 * place over levels [minlevel, maxlevel]. */
WC_API void RcpuThreshold(double* x, double* xmod, int* len, int* nlevels, int* ttype,
                   int* filter, int* filterlen, double* thresh, int* hardness,
                   int* minlevel, int* maxlevel);

/* rfunctions.cu:71 (RcpuSmooth).  Forward transform, threshold, inverse; x is
 * replaced by the smoothed signal.  *thresh is input for MANUAL and receives
 * the threshold used for UNIV and CV. */
WC_API void RcpuSmooth(double* x, int* len, int* nlevels, int* ttype, int* filter,
                int* filterlen, int* threshtype, double* thresh, int* hardness,
                int* minlevel, int* maxlevel, double* tol);

/* rfunctions.cu:102 (RgpuSmooth).  Same contract as RcpuSmooth; unlike the
 * reference it also accepts UNIV and the D4/C6/LA8 filters. */
WC_API void RgpuSmooth(double* x, int* len, int* nlevels, int* ttype, int* filter,
                int* filterlen, int* threshtype, double* thresh, int* hardness,
                int* minlevel, int* maxlevel, double* tol);

/* ---- .C glue with a status (R's .C passes only pointers to vector
 * elements; the wc_* calls below take scalars by value and structs).  Each
 * writes WC_OK or an error code to *status and prints nothing.  No
 * counterpart in the reference, whose symbols return no status
 * (rfunctions.cu:3-137). */

/* wc_transform through pointers: rfunctions.cu:21 (RgpuTransform) plus an
 * explicit precision and a status. */
WC_API void wc_transform_R(double* x, double* xmod, int* len, int* sense, int* nlevels,
                           int* ttype, int* filter, int* precision, int* status);
/* wc_threshold through pointers: rfunctions.cu:59 (RcpuThreshold) plus a
 * status. */
WC_API void wc_threshold_R(double* x, double* xmod, int* len, int* nlevels, int* ttype,
                           int* filter, double* thresh, int* hardness, int* minlevel,
                           int* maxlevel, int* status);
/* wc_smooth through pointers: rfunctions.cu:102 (RgpuSmooth) plus an
 * explicit precision and a status. */
WC_API void wc_smooth_R(double* x, int* len, int* nlevels, int* ttype, int* filter,
                        int* threshtype, double* thresh, int* hardness, int* minlevel,
                        int* maxlevel, double* tol, int* precision, int* status);
/* Batched smoothing in flat .C form -- the role of the reference's list API
 * RgpuTransformList (rfunctions.cu:139-154, a .Call placeholder whose R
 * wrapper is commented out at rfunctions.R:614-643).  Signal i occupies
 * data[offset[i] .. offset[i] + len[i]) (0-based; *total values in all) and
 * is described by element i of the parallel vectors (codes as for
 * RgpuSmooth).  thresh[i]: manual threshold in, threshold applied out;
 * iterations, kept, zeroed (may be NULL): CV iterations and kept/zeroed
 * detail counts out.  One persistent launch smooths every signal
 * (wc_smooth_batch). */
WC_API void RgpuSmoothBatch(double* data, int* total, int* nsig, int* offset, int* len,
                            int* nlevels, int* ttype, int* filter, int* threshtype,
                            double* thresh, int* hardness, int* minlevel, int* maxlevel,
                            double* tol, int* precision, int* iterations, int* kept,
                            int* zeroed, int* status);

/* ------------------------------------------------ 2. status-returning API */

/* Text of the last error on this thread ("" when none). */
WC_API const char* wc_last_error(void);

/* Maximum level count for (len, filterlen): check_len_levels,
 * wavutils.cpp:48-64 (0 when len is not a power of two >= filterlen). */
WC_API int wc_max_levels(int64_t len, int filterlen);

/* Process default precision used by the reference symbols (initially
 * WC_F64_EXACT, or the WAVECUDA_PRECISION environment variable: "exact",
 * "fast" or "fp32" -- fp32 converts at the boundary). */
WC_API int wc_set_default_precision(int precision);
WC_API int wc_get_default_precision(void);

/* Host-buffer transform (replaces RgpuTransform, rfunctions.cu:21-56, with a
 * status).  For WC_F32 the host data are still doubles; they are converted
 * on the device. */
WC_API int wc_transform(double* x, double* xmod, int64_t len, int sense, int nlevels,
                 int ttype, int filter, int precision);

/* Host-buffer threshold (replaces RcpuThreshold, rfunctions.cu:59-69). */
WC_API int wc_threshold(double* x, double* xmod, int64_t len, int nlevels, int ttype,
                 int filter, double thresh, int hardness, int minlevel,
                 int maxlevel);

/* Details of one smoothing call. */
typedef struct {
  double thresh;        /* threshold applied to the full transform */
  double thresh_univ;   /* universal threshold (the CV bracket's upper end) */
  int cv_iterations;    /* golden-section iterations (CV only) */
  int levels;           /* level count used */
  int64_t kept;         /* detail coefficients in [minlevel,maxlevel] kept */
  int64_t zeroed;       /* ... and set to zero (|c| < thresh) */
  double min_margin;    /* smallest |m1-m2|/m1 the search compared (CV) */
} wc_smooth_info;

/* Host-buffer smoothing (replaces RgpuSmooth/RcpuSmooth, rfunctions.cu:71-137,
 * with a status).  info may be NULL. */
WC_API int wc_smooth(double* x, int64_t len, int nlevels, int ttype, int filter,
              int threshtype, double* thresh, int hardness, int minlevel,
              int maxlevel, double tol, int precision, wc_smooth_info* info);

/* ---- batched smoothing: many signals of uneven length, filter, transform
 * and level count smoothed by one persistent launch.  The shape of the
 * reference's (placeholder) list API RgpuTransformList, rfunctions.cu:139-154,
 * in flat .C-friendly form: signals live back to back in one FP64 array and
 * are described by wc_signal records. */
typedef struct {
  int64_t offset;   /* first element of the signal in the data array */
  int64_t len;      /* power of two */
  int nlevels;      /* 0 = maximum */
  int ttype;        /* DWT 0 / MODWT 1 */
  int filter;       /* 1..4 */
  int threshtype;   /* MANUAL 0 / UNIV 1 / CV 2 */
  int hardness;     /* HARD 0 / SOFT 1 */
  int minlevel, maxlevel;
  double thresh;    /* threshold for MANUAL */
  double tol;       /* CV tolerance */
} wc_signal;

typedef struct {
  double thresh;        /* threshold applied */
  double thresh_univ;   /* universal threshold (CV bracket) */
  double min_margin;    /* smallest |m1-m2|/m1 the CV search compared */
  int iterations;       /* CV golden-section iterations */
  int status;           /* WC_OK */
  int64_t kept, zeroed; /* detail counts in [minlevel, maxlevel] */
} wc_signal_result;

typedef struct wc_batch_plan_s* wc_batch_plan;

/* Validates the signals, orders the work queue largest-first, sizes the
 * per-CTA scratch and allocates the plan's device buffers.  When a few long
 * CV searches would otherwise run on after the rest of the batch, the
 * longest are each split over two CTAs (one half-signal inverse each per
 * golden step, same results); the environment variable
 * WAVECUDA_BATCH_PAIRS=0 turns this off. */
WC_API int wc_batch_plan_create(const wc_signal* signals, int nsig, int precision,
                                wc_batch_plan* plan);
WC_API int wc_batch_plan_destroy(wc_batch_plan plan);
WC_API int wc_batch_plan_info(wc_batch_plan plan, int* grid, size_t* scratch_bytes);
/* Number of signals whose CV search the plan splits over two CTAs. */
WC_API int wc_batch_plan_pairs(wc_batch_plan plan, int* npairs);
/* Times a few grid sizes on a scratch copy of data (device) and keeps the
 * fastest; data is not modified.  Plans created later in the process (and
 * wc_smooth_batch) start from the grid found, for the same precision. */
WC_API int wc_batch_autotune(wc_batch_plan plan, const double* data, float* best_ms);
/* Smooths every signal of data (device, FP64) in place: one CUDA-graph launch
 * of the queue reset and the persistent kernel, asynchronous on stream. */
WC_API int wc_batch_run_device(wc_batch_plan plan, double* data, void* stream);
/* Copies the per-signal results to the host (synchronises stream). */
WC_API int wc_batch_results(wc_batch_plan plan, wc_signal_result* results, void* stream);
/* Host-buffer convenience: plan, copy in, run, copy out, results. */
WC_API int wc_smooth_batch(double* data, int64_t total, const wc_signal* signals, int nsig,
                           int precision, wc_signal_result* results);

/* ---- device-pointer API: inputs and outputs already in HBM.  stream is a
 * cudaStream_t (NULL = the library's own stream).  Calls are asynchronous
 * with respect to the host unless stated; scratch comes from the library's
 * per-device workspace (grown on demand, kept until wc_release()). */

/* DWT, out of place: in and out are distinct buffers of len elements (double
 * for the FP64 precisions, float for WC_F32).  FWD: in = signal, out =
 * interleaved transform.  BWD: in = interleaved transform, out = signal. */
WC_API int wc_dwt_device(const void* in, void* out, int64_t len, int sense,
                  int nlevels, int filter, int precision, void* stream);

/* Allocation-free DWT.  No counterpart in the reference: an addition for
 * callers that cannot let this library call cudaMalloc -- a host framework
 * that has reserved nearly all device memory for its own pool, or a
 * latency-critical loop that must not hit the synchronisation cudaFree
 * brings when a workspace grows.  Same arguments and results as
 * wc_dwt_device, but the scratch (coarse coefficients between passes and the
 * status word) lives in one fixed 1 MiB + 256 B device array compiled into
 * the library, which every GPU that loads it holds until the process exits.
 * Limit: len <= 2^22 samples (longer lengths are rejected with WC_ERR_ARG).
 * The first call on a device looks up the array's device address for that
 * device; make it before any stream capture (later calls look it up again
 * unless their stream is capturing).  All calls share the array and it keeps
 * the last call's contents, so calls that overlap on the GPU race.  Its
 * status word is sticky: a bounded wait that gave up sets bit 0, and
 * wc_device_status() (which allocates nothing) reads and clears it.
 * stream NULL means the legacy default stream (other wc_* calls given NULL
 * use the library's non-blocking stream, which is not ordered with it, so
 * pass the same explicit stream when mixing them).  Calls no cudaMalloc or
 * cudaFree. */
WC_API int wc_dwt_device_noalloc(const void* in, void* out, int64_t len, int sense,
                                 int nlevels, int filter, int precision, void* stream);

/* First-pass tiling of the DWT per (filter, precision): tile (power of two,
 * 256..16384 values per CTA), g0 (levels fused in the first pass), threads
 * (256 or 512 per CTA) and pipelined (1: persistent CTAs with double-buffered
 * bulk copies).  wc_tune_dwt times every candidate on a 2^log2n-sample signal
 * (forward + inverse) and keeps the fastest; the setting is per process. */
WC_API int wc_set_dwt_tiling(int filter, int precision, int tile, int g0, int threads,
                             int pipelined);
WC_API int wc_get_dwt_tiling(int filter, int precision, int* tile, int* g0, int* threads,
                             int* pipelined);
WC_API int wc_tune_dwt(int filter, int precision, int log2n, float* best_ms);

/* Tiling of the MODWT level kernels per (filter, precision): values a tile
 * aims at (a power of two in [256, 16384]) and the shared-memory budget per
 * CTA (16..200 KB), for the forward and the inverse kernels.  wc_tune_modwt
 * times every candidate on a 2^log2n-sample signal with nlevels levels and
 * keeps the fastest per direction; the setting is per process.  No
 * counterpart in the reference. */
WC_API int wc_set_modwt_tiling(int filter, int precision, int fwd_target, int fwd_smem_kb,
                               int inv_target, int inv_smem_kb);
WC_API int wc_get_modwt_tiling(int filter, int precision, int* fwd_target, int* fwd_smem_kb,
                               int* inv_target, int* inv_smem_kb);
WC_API int wc_tune_modwt(int filter, int precision, int log2n, int nlevels, float* fwd_ms,
                         float* inv_ms);
/* Levels the inverse MODWT fuses per launch (2 or 3; 0 restores the
 * filter's default: 3 for Haar, 2 otherwise).  More levels per launch move
 * the intermediate scaling sequence through HBM fewer times but stage a
 * deeper halo; wc_tune_modwt chooses it along with the tiling. */
WC_API int wc_set_modwt_inv_levels(int filter, int precision, int levels);
WC_API int wc_get_modwt_inv_levels(int filter, int precision, int* levels);
/* Levels the forward MODWT fuses per launch on the 16-byte tiles (1, 2 or 3;
 * 0 restores the default, 2; launches that fall back to the one-value tiles
 * fuse at most 2).  wc_tune_modwt chooses it along with the tiling. */
WC_API int wc_set_modwt_fwd_levels(int filter, int precision, int levels);
WC_API int wc_get_modwt_fwd_levels(int filter, int precision, int* levels);
/* 1 (the default): MODWT level kernels whose tiles allow it (one column, or
 * a multiple of 16 bytes of columns, and 16-byte aligned buffers) stage,
 * load and store 16 bytes per instruction; 0: every launch uses the
 * one-value-per-instruction tiles.  Both give bit-identical results.  No
 * counterpart in the reference. */
WC_API int wc_set_modwt_vector(int enable);

/* Time-ordered MODWT.  FWD: x (len) -> xmod (2*len*J).  BWD: xmod -> x.
 * BWD reads only s_J and d_1..d_J. */
WC_API int wc_modwt_device(void* x, void* xmod, int64_t len, int sense, int nlevels,
                    int filter, int precision, void* stream);

/* Exact median and MAD (1.4826 * median |x - median|) of n FP64 values in
 * device memory, as median()/mad() of utils.cpp:166-203 compute them (the
 * two middle order statistics averaged).  Synchronous; results on the host. */
WC_API int wc_median_mad_device(const double* data, int64_t n, double* median, double* mad,
                                void* stream);

/* ((0 + v[0]) + v[1]) + ... + v[n-1], every addition rounded as a serial
 * FP64 loop rounds it, for n non-negative FP64 terms in device memory
 * (the summation of the cross-validation loss, thresh.cpp:363-383).
 * Computed in parallel; synchronous; the sum is returned on the host. */
WC_API int wc_sequential_sum_device(const double* terms, int64_t n, double* sum, void* stream);

/* ---- coefficient extraction and formatting (R/rplotting.R:10-46,
 * R/rfunctions.R:925-1004), for large n on the device.  ttype 0 DWT
 * (interleaved, len values) or 1 time-ordered MODWT (2*nlevels*len values);
 * len a power of 2, 1 <= nlevels <= log2(len). */

/* getCoeffLevel(xw, level, coeffType) (rplotting.R:10-46): the 1-based
 * indices of the coefficients of `level` (1..nlevels); coeff_type 1 details
 * ("d"), 0 scaling ("s", DWT: level == nlevels only).  DWT: 2^(level-1)*d + 1
 * step 2^level; MODWT: 1..len whatever the level, as the reference returns.
 * Host arithmetic; idx may be NULL to query *count. */
WC_API int wc_coeff_level_indices(int64_t len, int nlevels, int ttype, int level, int coeff_type,
                                  int64_t* idx, int64_t capacity, int64_t* count);

/* Rows of WSTtoDT(xw, scaling, forPlotting = FALSE) (rfunctions.R:925-1004):
 * len (DWT) or 2*nlevels*len (MODWT) with scaling != 0, and without the
 * scaling rows len - len/2^nlevels or nlevels*len. */
WC_API int wc_wst_table_rows(int64_t len, int nlevels, int ttype, int scaling, int64_t* rows);

/* The WSTtoDT columns, in its row order: W (the coefficient), Level,
 * Translate and CoeffType (0 "s", 1 "d"); any column pointer may be NULL.
 * The per-level min/max placeholder rows of forPlotting = TRUE are not
 * produced.  Device pointers, enqueued on `stream`. */
WC_API int wc_wst_table_device(const double* w, int64_t len, int nlevels, int ttype, int scaling,
                               double* W, int32_t* level, double* translate, uint8_t* type,
                               void* stream);
/* The same with host arrays (copies in and out included; synchronous). */
WC_API int wc_wst_table(const double* w, int64_t len, int nlevels, int ttype, int scaling,
                        double* W, int32_t* level, double* translate, uint8_t* type);

/* ---- differentiation (no counterpart in the reference; backward calls for
 * gradient-based threshold tuning).  FP64 device vectors; `sense` names the
 * operator whose adjoint is applied (1 = the forward transform, 0 = the
 * inverse), so gin is the cotangent of that operator's output and gout the
 * cotangent of its input. */

/* DWT: adjoint(forward) is the inverse and adjoint(inverse) the forward
 * (the periodic orthonormal DWT is its own transpose pair). */
WC_API int wc_dwt_adjoint_device(const void* gin, void* gout, int64_t len, int sense, int nlevels,
                                 int filter, int precision, void* stream);

/* Time-ordered MODWT (FP64).  sense 1: gxmod (2*nlevels*len cotangents of
 * every stored block, s_l and d_l of each level) -> gx (len).  sense 0: gx
 * (cotangent of a reconstruction) -> gxmod (cotangents of s_J and d_1..d_J;
 * zero for the intermediate s blocks, which the inverse does not read). */
WC_API int wc_modwt_adjoint_device(double* gx, double* gxmod, int64_t len, int sense, int nlevels,
                                   int filter, void* stream);

/* Soft thresholding with one threshold per level (lambda: host array of
 * nlevels values, levels [minlevel, maxlevel], 0-based) on a DWT
 * (ttype 0) or MODWT (ttype 1) coefficient vector `coef`.  Given the
 * cotangent `gout` of the thresholded vector, writes gcoef (optional, same
 * length) and glambda (device, nlevels values, overwritten):
 * d eta/dc = 1{|c| >= t}, d eta/dt = -sign(c) 1{|c| >= t}. */
WC_API int wc_soft_threshold_adjoint_device(const double* coef, const double* gout, double* gcoef,
                                            double* glambda, int64_t len, int nlevels, int ttype,
                                            const double* lambda, int minlevel, int maxlevel,
                                            void* stream);

/* Loss of per-level soft thresholds and its gradient, for one FP64 signal x
 * (device).  lambda and grad are host arrays of nlevels values (levels
 * outside [minlevel, maxlevel] get gradient 0).
 *   WC_LOSS_SURE: Stein's unbiased risk estimate of the smoothed signal,
 *     ||f - x||^2 - n sigma^2 + 2 sigma^2 div f, where the divergence counts
 *     kept coefficients weighted by the per-level trace of synthesis times
 *     analysis (1 for the DWT, 2^-(l+1) for the MODWT).  The kept indicator
 *     is replaced by a logistic step of width eps (eps 0: the indicator, whose
 *     derivative is 0).  sigma <= 0: estimated as the MAD of the finest
 *     details; the value used is returned in *sigma_used (optional).
 *   WC_LOSS_CV: the two-fold cross-validation loss of interp_mse
 *     (thresh.cpp:344-385) with the even and odd halves transformed with
 *     nlevels-1 levels and half level l thresholded by lambda[l] for l in
 *     [minlevel, min(maxlevel, nlevels-2)].
 * Synchronous. */
#define WC_LOSS_SURE 0
#define WC_LOSS_CV 1
WC_API int wc_loss_grad(const double* x, int64_t len, int nlevels, int filter, int ttype,
                        int loss_type, const double* lambda, int minlevel, int maxlevel,
                        double sigma, double eps, double* loss, double* grad, double* sigma_used,
                        void* stream);

/* Per-level soft-threshold tuning by gradient descent for a batch of nsig
 * equal-length signals, all in one persistent launch (one CTA per signal
 * at a time).  No counterpart in the reference: it fits one threshold per
 * level, lambda_l = sigma u_l, to the SURE or the two-fold CV loss defined
 * for wc_loss_grad, by `iterations` Adam steps on u through the adjoint
 * kernels, keeps the best thresholds seen and (smooth != 0) overwrites each
 * signal with its soft-thresholded reconstruction.  CV thresholds fitted on
 * the half-length signals are rescaled by 1/sqrt(1 - log 2 / log len) for the
 * full signal (thresh.cpp:326) and levels above nlevels-2 take the level
 * nlevels-2 value.  Bulk arithmetic in `precision` (WC_F32, or WC_F64_FAST:
 * FP64 data with double-float arithmetic); loss and gradient totals in FP64. */
#define WC_FIT_MAX_LEVELS 24
typedef struct {
  int loss_type;          /* WC_LOSS_SURE or WC_LOSS_CV */
  int minlevel, maxlevel; /* thresholded levels (0-based); maxlevel < 0: nlevels-1 */
  int iterations;         /* Adam steps (the loss is evaluated iterations+1 times) */
  double step;            /* Adam step in units of sigma, e.g. 0.1 */
  double eps;             /* SURE: logistic width of the kept indicator in units of
                             sigma (0: the indicator itself) */
  double sigma;           /* noise level; <= 0: MAD of the finest details, per signal */
  const double* lambda0;  /* nlevels starting thresholds, or NULL: sigma sqrt(2 log len) */
  int precision;          /* WC_F32 or WC_F64_FAST */
  int smooth;             /* 1: overwrite x with the smoothed signals */
} wc_fit_opts;
typedef struct {
  double lambda[WC_FIT_MAX_LEVELS]; /* thresholds for the full signal (0 outside the range) */
  double grad0[WC_FIT_MAX_LEVELS];  /* loss gradient at the starting thresholds */
  double loss0, loss, sigma;        /* loss at the start, best loss, sigma used */
  int iterations, status;           /* status 1: not tunable (e.g. sigma 0) */
} wc_fit_result;
/* x: device, nsig * len FP64 values (signal k at x + k*len); results: host,
 * nsig records.  Synchronous. */
WC_API int wc_fit_thresholds_device(double* x, int64_t len, int nsig, int nlevels, int filter,
                                    int ttype, const wc_fit_opts* opts, wc_fit_result* results,
                                    void* stream);
/* Same with x in host memory (copied in and, when smoothing, back out). */
WC_API int wc_fit_thresholds(double* x, int64_t len, int nsig, int nlevels, int filter, int ttype,
                             const wc_fit_opts* opts, wc_fit_result* results);

/* ---- runtime helpers (device memory, pinned host memory, timing) */
WC_API int wc_device_count(int* count);
WC_API int wc_malloc_device(void** ptr, size_t bytes);
WC_API int wc_free_device(void* ptr);
WC_API int wc_malloc_host(void** ptr, size_t bytes); /* pinned */
WC_API int wc_free_host(void* ptr);
WC_API int wc_memcpy(void* dst, const void* src, size_t bytes, void* stream); /* any direction, async */
WC_API int wc_memset_device(void* ptr, int value, size_t bytes, void* stream);
WC_API int wc_stream_synchronize(void* stream);
WC_API int wc_default_stream(void** stream);
WC_API int wc_event_create(void** event);
WC_API int wc_event_destroy(void* event);
WC_API int wc_event_record(void* event, void* stream);
WC_API int wc_event_elapsed_ms(void* start, void* stop, float* ms);
/* Live per-kernel timing.  Between wc_profile_start() and wc_profile_stop()
 * the library brackets each of its kernel launches with CUDA events on the
 * launch's own stream; stop synchronises and returns, per kernel name, the
 * number of launches and their summed device time. */
typedef struct {
  char name[64];
  int64_t launches;
  double total_ms;
} wc_kernel_time;
WC_API int wc_profile_start(void);
WC_API int wc_profile_stop(wc_kernel_time* out, int capacity, int* count);

/* Reads and clears the current device's status words after synchronising
 * the device: the workspace word of the device-pointer calls and the word of
 * wc_dwt_device_noalloc.  Bit 0 set means a bounded device-side wait
 * (bulk-copy barrier) gave up and the kernel that waited skipped its work.
 * 0 when all is well.  Allocates nothing.  (The host-buffer calls and the
 * reference symbols read the workspace word themselves after their work: they
 * return WC_ERR_TIMEOUT -- the reference symbols print it -- and leave the
 * caller's buffers untouched, except a long DWT streamed in place over the
 * host link, which has already written part of x.) */
WC_API int wc_device_status(unsigned int* status);

/* ---- test hooks.  Failure injection without a GPU fault: the library's
 * allocation failures and its bounded waits can be made to happen on
 * purpose, so that their error paths can be tested. */
/* Every workspace slot that would have to grow beyond `bytes` fails with
 * WC_ERR_NOMEM instead of calling cudaMalloc (0 removes the cap). */
WC_API int wc_debug_set_workspace_cap(size_t bytes);
/* Bytes of device workspace the library holds on the current device. */
WC_API int wc_debug_workspace_bytes(size_t* bytes);
/* Launches one small kernel that arms an mbarrier for 16 bytes which no copy
 * delivers, so the library's bounded wait gives up after `polls` polls
 * (1..2^20) and records a timeout in a status word: target 0 the workspace
 * word, 1 the word of wc_dwt_device_noalloc.  Asynchronous; read the result
 * with wc_device_status() or through the next host-buffer call. */
WC_API int wc_debug_wait_probe(int target, unsigned int polls, void* stream);

/* Measured FP64 add/multiply throughput of the current device, in billions
 * of separately rounded FP64 operations per second (a short kernel of
 * independent multiply-add chains, never contracted to FMA, timed with CUDA
 * events): the arithmetic roofline of the WC_F64_EXACT kernels, which issue
 * exactly such operations.  Synchronous. */
WC_API int wc_measure_fp64_rate(double* gops, void* stream);

/* Number of kernels this library launched in this process so far. */
WC_API int64_t wc_kernel_launch_count(void);
/* Frees the workspace, streams and events the library holds. */
WC_API int wc_release(void);

#ifdef __cplusplus
}
#endif
#endif
