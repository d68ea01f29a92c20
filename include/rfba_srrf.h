/*
 * rfba_srrf.h — C-ABI of the GB300 SRRF radiality library (librfba_srrf.so).
 *
 * Drop-in replacement for RFBA's GradientCalc library. Three groups of entry
 * points:
 *
 *  1. The reference's own exports, same names, same signatures, same meaning:
 *       SRRFGradientCalc      RFBA Main/GradientCalc/GradientCalc.h:4, GradientCalc.cpp:169-173
 *       SRRFGetMag            RFBA Main/GradientCalc/GradientCalc.h:5, GradientCalc.cpp:176-178
 *       SRRFGradientCalcGPU   RFBA Main/GradientCalc/kernel.cuh:26,    kernel.cu:560-657
 *     They read ./SRRF.ini like the reference (sections [SRRF], [Temproal],
 *     [Radiality], [Weighting], optional [Split]), run synchronously on the
 *     current CUDA device with host buffers, and return 0 on success. Unlike the
 *     reference they return a negative rfba_status on failure (the reference
 *     always returns 0) and never abort the process.
 *
 *  2. An extended, stream-ordered interface on an explicit configuration
 *     (per-axis magnification, uint16 or float input, host or device pointers,
 *     explicit block lists, forward/backward pair). It replaces the reference's
 *     per-call cudaMalloc/cudaMemcpy driver (kernel.cu:560-657) and its serial
 *     per-block loop (GradientCalc.cpp:144-160).
 *
 *  3. Helpers: INI loading, block lists following GradientCalc.cpp:47-90 and
 *     the MATLAB doSplit.m rule, error text.
 *
 * Layouts (all little-endian, x fastest, as in the reference):
 *   input   [t][z][y][x]  (W*H*D*T elements; kernel.cu:36-40)
 *   output  [z][y][x] on the magnified grid (W*mx, H*my, D*mz), the layout of
 *           SRRF.raw (multispot5_place_methods.cc:272-274, 314).
 */
#ifndef RFBA_SRRF_H
#define RFBA_SRRF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1. Reference-compatible exports -------------------------------------- */

/* The reference's configuration record, field for field (kernel.cuh:3-24). */
typedef struct SRRFConf {
    float RingRadius;   /* ring radius, magnified voxels (default 0.5) */
    int Magnification;  /* integer magnification, all axes (default 5) */
    int AxesinRing;     /* ring has (2*AxesinRing)^2 samples (default 6) */
    int MainRange;
    int XRange;
    int YRange;
    int ZRange;
    int Method;         /* 0 TRM, 1 TRA, 2 TRPPM, 3 TRAC */
    int ITC;            /* integrate temporal correlations (TRAC) */
    int TRACOrder;      /* 2, 3 or 4 */
    int RemoveCon;      /* 1 clamps radiality at 0 */
    int Renormalize;
    int GradientSmooth;
    int IntensityW;
    int blockSizeX;
    int blockSizeY;
    int blockSizeZ;
} SRRFConf;

/* GradientCalc.cpp:169. imageDim = {W, H, D, T}. inImage: W*H*D*T floats,
 * outImage: W*H*D*mag^3 floats, both host memory owned by the caller. Splits
 * the volume into overlapping blocks (border 2, [Split] block sizes, default
 * 16) and pastes back each block's interior exactly like GradientCalc.cpp:
 * 92-116; all blocks run in one persistent kernel. Voxels the reference never
 * writes (the low border of 2*mag on each axis) are set to 0. */
int SRRFGradientCalc(float* inImage, int* imageDim, float* outImage);

/* GradientCalc.cpp:176-178: Magnification from ./SRRF.ini, default 5. */
int SRRFGetMag(void);

/* kernel.cu:560. One block (the whole input) with an explicit configuration;
 * host buffers; full magnified output. */
int SRRFGradientCalcGPU(float* inImage, int* imageDim, float* outImage, SRRFConf* conf);

/* ---- 2. Extended interface -------------------------------------------------- */

typedef enum rfba_status {
    RFBA_OK = 0,
    RFBA_ERR_INVALID = -1,     /* bad argument: null pointer, dims, config */
    RFBA_ERR_UNSUPPORTED = -2, /* valid but outside what the kernels handle */
    RFBA_ERR_NOMEM = -3,       /* device or host allocation failed */
    RFBA_ERR_CUDA = -4,        /* CUDA runtime error (text in rfba_last_error) */
    RFBA_ERR_TIMEOUT = -5,     /* a bounded device wait gave up */
    RFBA_ERR_IO = -6           /* file could not be read or written */
} rfba_status;

typedef enum rfba_dtype { RFBA_F32 = 0, RFBA_U16 = 1 } rfba_dtype;

/* Configuration. Field order mirrors SRRFConf with the magnification split per
 * axis (the reference's single Magnification is mag[0]=mag[1]=mag[2]). */
typedef struct rfba_srrf_config {
    float ring_radius;
    int mag[3];
    int axes_in_ring;
    int main_range, x_range, y_range, z_range;
    int method, itc, trac_order;
    int remove_con, renormalize, gradient_smooth, intensity_w;
    int block_size[3];
} rfba_srrf_config;

/* Pointer-location flags. */
#define RFBA_HOST_PTRS 0   /* in/out are host memory (pinned is fastest) */
#define RFBA_DEVICE_PTRS 1 /* in/out are device memory of the context's device */

/* One independent block of the input: the SRRF of the sub-volume
 * origin..origin+size (all time points), computed as if it were a whole image
 * (gradient clamps and interpolation windows at its own edges; kernel.cu:44-125,
 * 146). Only the magnified sub-region [lo, hi) (block-local fine coordinates) is
 * computed and written: element (x, y, z) of that region goes to
 * out[out_offset + (x-lo[0])*out_stride[0] + (y-lo[1])*out_stride[1]
 *         + (z-lo[2])*out_stride[2]]. */
typedef struct rfba_block {
    int32_t origin[3];
    int32_t size[3];
    int32_t lo[3];
    int32_t hi[3];
    int64_t out_offset;
    int64_t out_stride[3];
} rfba_block;

typedef struct rfba_ctx rfba_ctx; /* device, streams, scratch, plans, autotune cache */

/* Context on a CUDA device; scratch_budget_bytes caps the radiality stack (0 =
 * a default of a quarter of free device memory). */
int rfba_ctx_create(int device, size_t scratch_budget_bytes, rfba_ctx** out);
int rfba_ctx_destroy(rfba_ctx* ctx);

int rfba_srrf_config_default(rfba_srrf_config* cfg);        /* GradientCalc.cpp:19-41 */
int rfba_srrf_config_load_ini(const char* path, rfba_srrf_config* cfg); /* GradientCalc.cpp:15-42 */
int rfba_srrf_config_from_legacy(const SRRFConf* conf, rfba_srrf_config* cfg);

/* Whole volume as one block: out is the full magnified grid [D*mz][H*my][W*mx].
 * dims = {W, H, D, T}. stream is a cudaStream_t (NULL = the legacy default
 * stream, as everywhere in CUDA); with RFBA_HOST_PTRS the call returns when out
 * is written. Calls on one context share its scratch: a call on another stream
 * than the previous call is ordered after that call's work. */
int rfba_srrf_forward(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                      const int dims[4], float* out, int ptr_flags, void* stream);

/* Explicit block list (any sizes, any count) in one persistent launch. The
 * output pointer and every block's out_offset/out_stride address one array
 * of out_elems floats. */
int rfba_srrf_forward_blocks(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                             const int dims[4], const rfba_block* blocks, int nblocks, float* out,
                             int64_t out_elems, int ptr_flags, void* stream);

/* The same block list, one launch per block with its own host<->device copies,
 * as the reference's GradientCalc.cpp:144-160 loop does (the "plain" path).
 * Host pointers only. */
int rfba_srrf_forward_blocks_plain(rfba_ctx* ctx, const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                                   const int dims[4], const rfba_block* blocks, int nblocks, float* out,
                                   int64_t out_elems);

/* Whole-volume forward that allocates no device memory. No counterpart in the
 * reference. For callers that cannot call cudaMalloc where they need a map: an
 * acquisition loop that must not stall on cudaMalloc's device-wide
 * synchronisation, a host whose device memory belongs to its own pool, a plugin
 * environment that forbids device allocation. in and out are device pointers
 * of the current device, or managed memory (layouts as rfba_srrf_forward;
 * another GPU's memory is refused with RFBA_ERR_INVALID); all temporaries
 * live in one fixed 128 MiB
 * device array inside the library, which every GPU that loads the library holds
 * until the process exits. Volumes whose scratch (about 8 bytes per output
 * subvoxel per time point plus small tables) exceeds it are rejected with
 * RFBA_ERR_UNSUPPORTED and a message. The first call on a device looks the
 * array up (cudaGetSymbolAddress) and should come before any stream capture.
 * All calls share the array: calls that overlap on the GPU race, so serialise
 * them. Stream-ordered on `stream` (a cudaStream_t, NULL = the legacy default
 * stream); its tables and descriptors reach the array through small kernels
 * that carry them as launch parameters, so no host buffer is read after the
 * call returns. */
int rfba_srrf_forward_static_scratch(const rfba_srrf_config* cfg, const void* in, rfba_dtype dtype,
                                     const int dims[4], float* out, void* stream);

/* Differentiable pair (no counterpart in the reference, which has no
 * derivatives). Whole volume as one block, float32 device input [t][z][y][x].
 * shifts: device T x 3 floats (x, y, z per volume) or NULL. The forward first
 * resamples each volume at x + shifts[t] (Catmull-Rom, the reference's cubic of
 * kernel.cu:128-138, edge clamped, one axis at a time x, y, z) and then runs the
 * SRRF forward; out is the map as rfba_srrf_forward writes it.
 * The backward takes dL/dmap (device, map layout; NaN map voxels get no
 * gradient) and writes dL/din (T x D x H x W) and, if dL_dshift is not NULL,
 * dL/dshifts (T x 3). It covers every temporal method: TRM, TRA and TRPPM
 * (Methods 0-2; TRM's derivative goes to the first time point that reaches
 * the maximum) and TRAC with Integrate_Temporal_Correlations 0 or 1 (the
 * shipped setting; its backward always recomputes the stacks). It reuses the radiality stacks of the
 * last rfba_srrf_forward_shifted on the same context with the same
 * configuration, input and shifts when that forward held the whole series at
 * once, or the carried temporal state it kept when it ran in time batches
 * (TRAC with ITC 0, see rfba_ctx_set_time_batch); otherwise it runs that
 * forward itself. The interpolated gradient field is recomputed, not stored.
 * Stream-ordered. */
int rfba_srrf_forward_shifted(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                              const int dims[4], float* out, void* stream);
int rfba_srrf_backward(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                       const int dims[4], const float* dL_dmap, float* dL_din, float* dL_dshift, void* stream);
/* The same pair restricted to the fine region [lo, hi) of the magnified grid
 * (x, y, z; 0 <= lo < hi <= dims * mag per axis), for splitting one series'
 * map across processes (no counterpart in the reference). The forward writes
 * the region packed [z][y][x] into out; the backward takes dL/dregion in that
 * layout and writes the region's whole contribution to dL/din and dL/dshifts,
 * so the contributions of disjoint regions that tile the map sum to
 * rfba_srrf_backward's result. Region calls always recompute their stacks.
 * Stream-ordered. */
int rfba_srrf_forward_shifted_region(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in,
                                     const float* shifts, const int dims[4], const int lo[3], const int hi[3],
                                     float* out, void* stream);
int rfba_srrf_backward_region(rfba_ctx* ctx, const rfba_srrf_config* cfg, const float* in, const float* shifts,
                              const int dims[4], const int lo[3], const int hi[3], const float* dL_dregion,
                              float* dL_din, float* dL_dshift, void* stream);
/* CUDA-event duration of the last backward (with timing enabled). */
int rfba_ctx_last_backward_ms(rfba_ctx* ctx, double* ms);

/* Block lists. GradientCalc.cpp:47-116 (border 2, put-back into the full
 * magnified output, magnification per axis, the reference's single Mag when the
 * three are equal); returns the block count, or a
 * negative status. With blocks == NULL only counts. */
int rfba_blocks_gradientcalc(const rfba_srrf_config* cfg, const int dims[4], rfba_block* blocks, int cap);
/* doSplit.m (Matlab Scripts/doSplit.m:1-19) per axis with block edge max_size
 * and border; each block writes its whole magnified output into a packed array
 * (blocks in x-fastest order, each [z][y][x]). */
int rfba_blocks_dosplit(const rfba_srrf_config* cfg, const int dims[4], const int max_size[3], int border,
                        rfba_block* blocks, int cap, int64_t* out_elems);

/* Ring factorisation used by the kernels for this configuration: distinct ring
 * points (the reference evaluates all (2*AxesinRing)^2 samples, kernel.cu:215-
 * 216; coincident ones are merged with a multiplicity), distinct (x, y) pairs,
 * distinct x values, and the raw sample count. Any pointer may be NULL. */
int rfba_srrf_plan_info(const rfba_srrf_config* cfg, int* npoints, int* npairs, int* nxvalues, int* nraw);

/* ---- 3B spot likelihood (the localisation step downstream of the SRRF map) --- */

/* The model of RFBA's 3B step for one spot: a three-state chain (0 spot on,
 * 1 off, 2 bleached) with transition matrix A (row-major, [from][to]) and
 * initial probabilities pi (RFBA Main/multispot5.cfg:15-16), Gaussian pixel
 * noise of the given variance on the normalised intensities, the spot's z
 * scale (multispot5_headless.cc:180-181), and log-normal priors on brightness
 * and blur (storm.h:417-434). */
typedef struct rfba_3b_model {
    double A[9];
    double pi[3];
    double variance;
    double z_factor;
    double mu_brightness, sigma_brightness;
    double mu_blur, sigma_blur;
} rfba_3b_model;

/* SpotNegProbabilityDiffWithSampledBackground::operator() (RFBA Main/
 * multispot5.cc:616-664): the derivative of the negative log probability of
 * one spot (brightness, blur, x, y, z) with respect to its parameters, averaged
 * over S samples of the other spots' intensities, the function 3B's
 * conjugate-gradient spot optimiser evaluates. sample_bg [S][F][P] and
 * pixel_intensities [F][P] are doubles, pixels [P][3] the mask voxels (x, y, z);
 * host or device memory (ptr_flags). spot, out[5] and log_prob[S] (each
 * sample's log probability; may be NULL) are host memory; the call returns
 * when out is written. spot[0] <= 0 or spot[1] <= 0 gives NaN, as the
 * reference does; entries of A or pi outside [0, 1] give RFBA_ERR_INVALID.
 * FP64 throughout when log_prob is requested; without it (as the spot
 * optimisers call it) the per-frame sums over the pixels run in double-float
 * arithmetic on the FP32 pipe (about 2^-46 relative per operation) on
 * residuals staged once. */
int rfba_3b_spot_gradient(rfba_ctx* ctx, const rfba_3b_model* model, const double* sample_bg,
                          const double* pixel_intensities, const int* pixels, int S, int F, int P,
                          const double spot[5], double out[5], double* log_prob, int ptr_flags, void* stream);

/* The spot optimisation 3B runs on each spot after drawing its background
 * samples (RFBA Main/multispot5.cc:1614-1636): ConjugateGradientOnly<5>
 * (conjugate_gradient_only.h) from `spot`, steps limited per parameter by
 * `limit` (the reference's `limit` vector: cg.max_motion times
 * (brightness limit, 1, 1, 1, 1)), at most max_iterations line searches
 * (main.cg.max_iterations), with rfba_3b_spot_gradient's value as the gradient
 * on data staged once on the device. Writes the final spot; iterations and
 * evaluations (gradient calls) may be NULL. Same arguments, layouts and
 * synchronous return as rfba_3b_spot_gradient. */
int rfba_3b_optimise_spot(rfba_ctx* ctx, const rfba_3b_model* model, const double* sample_bg,
                          const double* pixel_intensities, const int* pixels, int S, int F, int P,
                          const double spot[5], const double limit[5], int max_iterations, double spot_out[5],
                          int* iterations, int* evaluations, int ptr_flags, void* stream);

/* The same optimiser on the host, with the gradient supplied by the caller
 * (fn returns 0, or a non-zero value that stops the run and is returned). No
 * device work; for optimisers whose gradient lives elsewhere and for checking
 * the optimiser itself. */
typedef int (*rfba_grad5_fn)(const double x[5], double grad[5], void* user);
int rfba_cg_only_run(const double start[5], const double limit[5], int max_iterations, rfba_grad5_fn grad,
                     void* user, double x_out[5], int* iterations, int* evaluations);

/* get_spot_pixels (RFBA Main/multispot5.cc:1001-1020) for K spots: the mask of
 * spot k is every pixel whose position equals the spot's rounded centre
 * (half away from zero) plus an offset of getBall(blur * 6 + 1)
 * (multispot5.cc:1259-1272), in the ball's order; pixels [P][3] (x, y, z) must
 * be sorted by (z, y, x) as the reference's pixel list is. Writes
 * mask_offsets[K + 1] and, when mask_pixels is not NULL, up to cap pixel
 * indices; *nnz receives the total. Host memory, no device work. */
int rfba_3b_spot_masks(const int* pixels, int P, const double* spots, int K, int* mask_offsets, int* mask_pixels,
                       long long cap, long long* nnz);

/* GibbsSampler2 (RFBA Main/sampled_multispot.h:360-690) on the GPU: a fresh
 * sampler (every spot off in every frame) draws n_draws samples, each after
 * `sweeps` passes over the spots (main.gibbs.samples and gibbs.mixing_iterations
 * in multispot5.cfg). Per spot: remove it over its mask where it is on, the
 * frames' log probabilities with it on and off over the mask, the 3-state
 * forward filter, a backward draw of its states, add it back. Spot k's
 * intensity is spot_shape at every pixel (storm.h:229-235, model->z_factor);
 * masks as rfba_3b_spot_masks writes them (mask_offsets[K + 1], mask_pixels).
 * pixel_intensities [F][P], pixels [P][3], spots [K][5] (brightness, blur, x,
 * y, z). Outputs (either may be NULL): states [n_draws][K][F] (0 on, 1 off,
 * 2 bleached) and sample_intensities [n_draws][F][P], the sampler's
 * intensities after each draw (sampled_multispot.h:684-689); with
 * exclude_spot = s >= 0 spot s's intensity is taken off every pixel of the
 * frames where it is on, as multispot5.cc:1606-1608 does before the spot
 * optimiser uses the draws as background samples. Random numbers:
 * Philox4x32-10 keyed by seed (the reference's distribution, not its MT19937
 * stream). 1 <= F <= 2048. Synchronous. */
int rfba_3b_gibbs_sample(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities, const int* pixels,
                         const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                         int sweeps, int n_draws, unsigned long long seed, int exclude_spot, uint8_t* states,
                         double* sample_intensities, int ptr_flags, void* stream);

/* One sweep of the sampler above from all spots off, with what each spot's
 * draw was made from: log_prob [K][F][2] the frame's log probability with the
 * spot on and off (SpotWithBackgroundMasked, spot_with_background.hh:98-137)
 * and filtered [K][F][3] the forward filter's state distribution per frame
 * (forward_algorithm_delta2, forward_algorithm.h:385-431, normalised), given
 * the states the sweep drew for the spots before it; states [K][F]. Any output
 * may be NULL. Synchronous. */
int rfba_3b_gibbs_trace(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities, const int* pixels,
                        const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                        unsigned long long seed, uint8_t* states, double* log_prob, double* filtered, int ptr_flags,
                        void* stream);

/* NegativeFreeEnergy::compute_with_mask (RFBA Main/multispot5.cc:335-405): the
 * model's negative free energy by slow-growth thermodynamic integration, the
 * Gibbs sampler above drawing `samples` times (add_remove.thermo.samples) with
 * the noise variance grown as variance_from_sample and the derivative by a
 * five-point stencil, plus the log-normal priors; *value is what
 * compute_with_mask returns. residuals [samples] (may be NULL) receives each
 * draw's sum of squared residuals over all frames and pixels. Synchronous. */
int rfba_3b_free_energy(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities, const int* pixels,
                        const double* spots, const int* mask_offsets, const int* mask_pixels, int K, int F, int P,
                        int samples, int sweeps, unsigned long long seed, double* value, double* residuals,
                        int ptr_flags, void* stream);

/* rfba_3b_free_energy for nmodels (1 or 2) models of one block side by side,
 * their Gibbs chains in one launch (a model comparison, which the reference
 * runs on two threads, multispot5.cc:2096-2108): model i has K[i] spots
 * spots[i] [K[i]][5] with masks mask_offsets[i] / mask_pixels[i] and its own
 * seed; values[i] is what compute_with_mask returns. Each model's value equals
 * rfba_3b_free_energy's with the same seed. Host memory. Synchronous. */
int rfba_3b_free_energy_models(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities,
                               const int* pixels, int F, int P, int nmodels, const double* const* spots, const int* K,
                               const int* const* mask_offsets, const int* const* mask_pixels, int samples, int sweeps,
                               const unsigned long long* seeds, double* values);

/* One pass of FitSpots::optimize_each_spot_in_turn_for_several_passes (RFBA
 * Main/multispot5.cc:1511-1690), the main loop of a 3B block fit, on the GPU:
 * the spots (spots [*nspots][5], host, updated in place) are ordered by
 * position as pass `pass` orders them (x ascending, x descending, then y
 * descending; the reference's third branch repeats "% 4 == 1" and is never
 * taken), their masks kept at their old places as the reference's reordering
 * leaves them (multispot5.cc:1570); then each spot in turn: a fresh Gibbs
 * sampler (rfba_3b_gibbs_sample) draws main_samples samples with `sweeps`
 * passes each, the spot is taken off them, ConjugateGradientOnly<5> optimises
 * it on rfba_3b_spot_gradient over those samples (at most cg_max_iterations
 * line searches, motion limits `limit`), its mask is recomputed, and it is
 * erased when the mask is empty or, with position_extra_radius >= 0, when its
 * rounded position leaves the pixels dilated by getBall(position_extra_radius)
 * (the position prior, multispot5.cc:1280-1290, 1653-1674); *nspots receives
 * the spots kept. Spot s's draws use the seed rfba_3b_pass_seed(seed, pass, s).
 * pixel_intensities [F][P] and pixels [P][3] (sorted by (z, y, x)) are host
 * memory; *evaluations (may be NULL) receives the gradient evaluations.
 * Synchronous. */
int rfba_3b_optimise_pass(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities,
                          const int* pixels, int F, int P, double* spots, int* nspots, int pass, int main_samples,
                          int sweeps, int cg_max_iterations, const double limit[5], double position_extra_radius,
                          unsigned long long seed, int* evaluations);
/* The Gibbs seed of spot s in pass `pass` of rfba_3b_optimise_pass. */
unsigned long long rfba_3b_pass_seed(unsigned long long seed, int pass, int s);

/* sampled_background_spot_hessian_ffbs (RFBA Main/multispot5.cc:824-985): the
 * Hessian of one spot's log probability with the other spots' intensities
 * sampled by the S draws sample_bg [S][F][P] (the spot taken off them, as
 * rfba_3b_gibbs_sample's exclude_spot gives them) and the spot's own states by
 * bs_iterations backward samples per draw of its forward-filtered on / off
 * chain (SpotWithBackground over all P pixels, spot_with_background.hh:
 * 98-150): the sum over samples of hess + deriv deriv^T over the frames where
 * the spot is on (hess = sum_p e H_p - g_p g_p^T, deriv = sum_p e g_p, e the
 * residual with the spot on, g_p and H_p the spot's gradient and Hessian at
 * pixel p, storm.h:87-146), divided by (bs_iterations S variance), less the
 * outer product of the mean derivative, plus the second derivatives of the
 * log-normal priors on brightness and blur (storm.h:446-449). hess[25]
 * (row-major, symmetric; the reference leaves its entry [4][3] unwritten) is
 * host memory. Random numbers: Philox4x32-10 keyed by seed. 1 <= F <= 2048,
 * bs_iterations >= 1. FP64. Synchronous. */
int rfba_3b_spot_hessian(rfba_ctx* ctx, const rfba_3b_model* model, const double* sample_bg,
                         const double* pixel_intensities, const int* pixels, int S, int F, int P,
                         const double spot[5], int bs_iterations, unsigned long long seed, double hess[25],
                         int ptr_flags, void* stream);

/* FreeEnergyHessian::hessian (RFBA Main/multispot5.cc:693-775), the "pure
 * MCMC" Hessian of the negative free energy with respect to spot `spot`: the
 * unmasked Gibbs sampler (GibbsSampler, sampled_multispot.h:240-330) draws
 * `samples` times (`sweeps` sweeps each) with every spot of spots [K][5] in
 * the model; per draw, over the frames where the spot is on, h = sum_p e H_p
 * - g_p g_p^T and d = sum_p e g_p with e the residual of the draw (which
 * holds the spot), plus the log-normal priors' derivatives; the result is
 * (sum h + sum d d^T) / (samples variance) less the outer product of
 * sum d / (samples variance), as the reference forms it. The reference's
 * modification step has this call commented out (multispot5.cc:2042-2043) in
 * favour of rfba_3b_spot_hessian; it is here for callers of the class.
 * Host memory; hess[25] row-major. Philox draws keyed by seed. Synchronous. */
int rfba_3b_free_energy_hessian(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities,
                                const int* pixels, const double* spots, int K, int F, int P, int spot, int samples,
                                int sweeps, unsigned long long seed, double hess[25]);

/* Settings of a 3B block fit (FitSpots, RFBA Main/multispot5.cc:1329-1505), the
 * reference's variable names and multispot5.cfg values in brackets. */
typedef struct rfba_3b_fit_params {
    int main_passes;             /* main.passes (4) */
    int main_samples;            /* main.gibbs.samples (10) */
    int main_cg_max_iterations;  /* main.cg.max_iterations (5) */
    int sweeps;                  /* gibbs.mixing_iterations (1) */
    int add_remove_tries;        /* add_remove.tries (10) */
    int opt_samples;             /* add_remove.optimizer.samples (20) */
    int opt_attempts;            /* add_remove.optimizer.attempts (10) */
    int opt_hess_inner_samples;  /* add_remove.optimizer.hessian_inner_samples (1000) */
    int h_outer_samples;         /* add_remove.hessian.outer_samples (100) */
    int h_inner_samples;         /* add_remove.hessian.inner_samples (1000) */
    int thermo_samples;          /* add_remove.thermo.samples (1000) */
    double limit[5];             /* cg.max_motion x (brightness limit, 1, 1, 1, 1) */
    double position_extra_radius; /* position.extra_radius (2.3); < 0: position.use_prior = 0 */
    /* add_guide = 1 (multispot5_headless.cc:177-179): proposed spots are drawn
     * from this SRRF map as InitGuide / GetPoint draw them (multispot5.cc:
     * 2164-2231; rfba_srrf_seed_spots' distribution over the pixels' subvoxels):
     * host memory [z][y][x], guide_dims its x, y, z extents, guide_mag the
     * magnification, in the pixels' coordinates (the SRRF.raw of the same
     * image). NULL: a uniform pixel plus a uniform offset. */
    const float* guide_map;
    int guide_dims[3];
    int guide_mag;
} rfba_3b_fit_params;

/* What one model modification did. */
typedef struct rfba_3b_modify_record {
    int added;        /* 1: a spot was proposed for addition; 0: one for removal */
    int kept;         /* 1: the model without the mobile spot, 2: with it */
    int zero_prior;   /* the optimised mobile spot left the allowed area */
    int bad_hessian;  /* the Hessian there was not negative definite: the original model kept */
    int evaluations;  /* gradient evaluations of the mobile spot's optimisation */
    double model1_energy, model2_energy;  /* -free energy of each model (when compared) */
    double occam;     /* -log(det(-H / 2 pi)) / 2, Laplace's approximation */
    double position_log_prior;  /* log prior of model 2 minus model 1 */
    double spot[5];   /* the optimised mobile spot */
} rfba_3b_modify_record;

/* One try of FitSpots::try_modifying_model (RFBA Main/multispot5.cc:1840-2160)
 * on the GPU. Model 1 is the spots without, model 2 with, a mobile spot: with
 * probability 1/2 (always when *nspots <= 1) a spot is proposed at a random
 * pixel plus a uniform offset in [-0.5, 0.5) per axis, with the modes of the
 * brightness and blur priors, else a random spot is proposed for removal. The
 * mobile spot is optimised on opt_samples GibbsSampler2 draws
 * (ConjugateGradientOnly<5>, at most 500 line searches per attempt); after
 * each attempt but the last the sampled-background Hessian
 * (rfba_3b_spot_hessian, opt_hess_inner_samples) is decomposed and, unless it
 * is negative definite, the optimiser restarts 0.1 along the eigenvector of its
 * fourth-smallest eigenvalue. A mobile spot outside the allowed area keeps
 * model 1 (with a guide map the proposal's position is drawn from the map
 * instead). Otherwise the Hessian is taken again on h_outer_samples draws of the
 * sampler over all pixels (GibbsSampler, sampled_multispot.h:240-330) with
 * h_inner_samples backward samples; when its negation's smallest eigenvalue is
 * above 1e-6, model 2 is kept if its negative free energy (rfba_3b_free_energy,
 * thermo_samples) plus -log(det(-H / 2 pi)) / 2 plus the position prior's log
 * ratio exceeds model 1's, and otherwise the original model is kept. spots
 * [capacity][5] (capacity >= *nspots + 1), pixel_intensities [F][P] and pixels
 * [P][3] (sorted by (z, y, x)) are host memory; *nspots receives the model
 * kept; record may be NULL. The proposal's random choices come from a
 * SplitMix64 stream of seed, the draws' from Philox4x32-10 with seeds mixed
 * from it. Eigenvectors are signed with their largest component positive (the
 * reference's LAPACK sign is not specified). Synchronous. */
int rfba_3b_modify_model(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities,
                         const int* pixels, int F, int P, double* spots, int* nspots, int capacity,
                         const rfba_3b_fit_params* params, unsigned long long seed, rfba_3b_modify_record* record);

/* Progress of rfba_3b_fit after each step of iteration `iteration`: step <
 * main_passes is the pass just finished, step >= main_passes the model
 * modification step - main_passes; spots [nspots][5] are the current ones. A
 * non-zero return stops the fit there (it returns RFBA_OK with those spots). */
typedef int (*rfba_3b_fit_fn)(int iteration, int step, const double* spots, int nspots, void* user);

/* FitSpots::run (RFBA Main/multispot5.cc:2234-2278) on the GPU: `iterations`
 * iterations from first_iteration, each main_passes passes
 * (rfba_3b_optimise_pass, ordered by pass + iteration as the reference orders
 * them) and add_remove_tries model modifications (rfba_3b_modify_model); a
 * modification is skipped when spots has no room for another spot. Arguments
 * as rfba_3b_modify_model; progress may be NULL. Synchronous. */
int rfba_3b_fit(rfba_ctx* ctx, const rfba_3b_model* model, const double* pixel_intensities, const int* pixels, int F,
                int P, double* spots, int* nspots, int capacity, const rfba_3b_fit_params* params,
                int first_iteration, int iterations, unsigned long long seed, rfba_3b_fit_fn progress, void* user);

/* The masks the library's unmasked sampler (GibbsSampler, used for the model
 * modification's Hessian draws and rfba_3b_free_energy_hessian) runs with:
 * each spot's support, the pixels where its Gaussian factor exp(-|x - mu|^2 /
 * (2 blur^2)), the z difference divided by z_factor, is at least 2^-60, in
 * pixel order. A frame's on - off log probability, the only part of it the
 * filter uses, then differs from the all-pixel sums' by less than 2^-60 of
 * the terms kept. Same outputs as rfba_3b_spot_masks. Host only. */
int rfba_3b_support_masks(const int* pixels, int P, const double* spots, int K, double z_factor, int* mask_offsets,
                          int* mask_pixels, long long cap, long long* nnz);

/* Host helpers of the model modification, exported for testing: eigenvalues
 * (ascending) and eigenvectors (rows, largest-magnitude component positive)
 * of a symmetric 5x5 matrix by cyclic Jacobi rotations, and the determinant of
 * a 5x5 matrix by Gaussian elimination with partial pivoting. No device work. */
int rfba_sym_eigen5(const double a[25], double evals[5], double evecs[25]);
double rfba_det5(const double a[25]);

/* Device-side failure check. No counterpart in the reference (GradientCalc.cpp
 * and kernel.cu check no CUDA status; every call returns 0). Waits for the
 * work the context last enqueued and reports failures its kernels recorded
 * since the last report: RFBA_ERR_TIMEOUT when a bounded device wait gave up
 * (an input staging copy that did not land within about a second), and, with
 * RFBA_CHECKS=1 in the environment, RFBA_ERR_CUDA for an out-of-range index.
 * Calls with host pointers report these themselves before they return;
 * device-pointer calls are asynchronous and report through this function. */
int rfba_ctx_check(rfba_ctx* ctx);

/* Measured FP32 FMA throughput of a device in TFLOP/s (a short probe kernel of
 * independent FMA chains on every SM, about 20 ms): the measured ceiling for the
 * radiality kernel's roofline. No counterpart in the reference (measurement). */
int rfba_probe_fp32_fma_peak(int device, double* tflops);

/* Measurement hooks: CUDA-event durations of the last call's kernels, taken on
 * the stream they were launched on (enable first), and the number of kernels
 * the context has launched. */
int rfba_ctx_set_timing(rfba_ctx* ctx, int enable);
int rfba_ctx_last_timing(rfba_ctx* ctx, double* radiality_ms, double* temporal_ms, long long* launches);
/* Launch overrides for tuning: CTAs of the radiality kernel and time points per
 * work item (0 = automatic). */
int rfba_ctx_set_launch(rfba_ctx* ctx, int grid, int t_chunk);
/* Time batches of rfba_srrf_forward / rfba_srrf_forward_blocks. A series whose
 * radiality and intensity stacks fit the context's scratch budget is reduced
 * whole; a longer one runs in batches of 25 volumes: the radiality of a batch
 * fills its stacks, then its values are folded into a per-subvoxel temporal
 * state carried to the next batch (TRM, TRA, TRPPM: the same sums in the same
 * order, maps bit-identical to the one-pass reduction; TRAC with ITC 0: the
 * cumulant window sums around the first batch's mean, combined in double at
 * the end, equal to rounding). The map is cut into z slices only where one
 * batch's stacks and the state still exceed the budget. TRAC with ITC 1 bins
 * the whole series and slices space instead. volumes > 0 forces batches of that
 * many volumes (rfba_srrf_backward then runs in batches too for TRA and TRAC
 * with ITC 0: per batch the radiality of the batch and of the TRAC order - 1
 * volumes on either side, its temporal adjoint from the carried state and its
 * radiality adjoint), < 0 turns batches off, 0 restores the automatic choice:
 * batches of 25 where the whole series' stacks exceed the budget; for TRAC with
 * ITC 0 rfba_srrf_forward_shifted then keeps every slice's carried state and the
 * rfba_srrf_backward that follows with the same arguments reuses it (without
 * one, the backward slices space). The
 * reference holds its whole series in memory (GradientCalc.cpp, one block at a
 * time); the batches correspond to streaming the series' frames through HBM. */
int rfba_ctx_set_time_batch(rfba_ctx* ctx, int volumes);
/* Volumes per batch and batches of the last forward (0, 0: one pass over the
 * whole series), and its spatial passes (z slices or groups of blocks whose
 * stacks fit the budget together; 1 when everything fit at once). */
int rfba_ctx_last_time_batches(rfba_ctx* ctx, int* volumes, int* batches, int* passes);
/* SRRF-guided spot seeding: replaces the rejection loops of
 * multispot5_place_methods.cc:291-341 (place_spots_intensity_sampled) and
 * multispot5.cc:2164-2231 (InitGuide / GetPoint). Candidates are the mag^3
 * subvoxels of each input voxel in `voxels` ([n][3] ints x, y, z, the 3B block
 * mask's pixels), weighted by the map value ([z][y][x] floats, map_dims = its
 * x, y, z extents, the SRRF.raw layout; NaN and negative values weigh 0, an
 * all-zero map weighs every candidate 1). Writes num_spots positions [n][3] in
 * input-voxel units, (subvoxel + U(-0.5, 0.5)) / mag per axis like the
 * reference. Drawn on the GPU by inverse CDF with a counter-based generator
 * keyed by `seed`: the reference's distribution, not its random stream.
 * Synchronous (returns when xyz is written). */
int rfba_srrf_seed_spots(rfba_ctx* ctx, const float* map, const int map_dims[3], int mag, const int* voxels,
                         int nvoxels, int num_spots, unsigned long long seed, float* xyz, int ptr_flags, void* stream);

/* CombineBlock (Matlab Scripts/CombineBlock.m, genpsf.m, loadResult.m): the
 * reconstruction from 3B's localisations. No counterpart in the reference's
 * compiled code (the reference does this in MATLAB).
 *
 * rfba_combine_psf: genpsf(sigma, crop_threshold) — uint16 PSF, [z][y][x],
 * psf_dims = x, y, z extents; returns the element count (PSF copied when cap
 * suffices, pass NULL/0 to query).
 * rfba_combine_load_result: loadResult.m on one res_i_j_k.txt — the spots
 * (intensity, blur, x, y, z as doubles) of every "PASS" line that lie strictly
 * inside the block minus its border (block_start 1-based, as doSplit.m).
 * rfba_combine_render: CombineBlock.m:24-173 on the spots of all blocks:
 * histogram on the zoom-times grid (round half away from zero), noise mask
 * (box sums of occupied voxels over (2r+1)^2 x (2rz+1) above noise_threshold in
 * the interior, kept at the borders), convn(..., psf, 'same') in 64-bit
 * integers, scaled to uint16 by the maximum. out: [Z*zoom][Y*zoom][X*zoom]
 * uint16 (host); dropped = spots that fell outside the grid. Synchronous. */
int rfba_combine_psf(double sigma, double crop_threshold, uint16_t* psf, long long cap, int psf_dims[3]);
int rfba_combine_load_result(const char* path, int border, const int block_start[3], const int block_size[3],
                             double* spots, long long cap, long long* nspots);
int rfba_combine_render(rfba_ctx* ctx, const double* spots, long long nspots, const int img_dims[3], int zoom,
                        const uint16_t* psf, const int psf_dims[3], int noise_r, int noise_rz, int noise_threshold,
                        uint16_t* out, long long* dropped);

/* Schedule of the last rfba_srrf_forward / rfba_srrf_forward_blocks call: tile
 * rows (tile shape), tile order (0 largest block first, 1 interleaved across
 * blocks), whether it was replayed as a CUDA graph, and whether this call ran
 * the autotuner. The extended forward autotunes the schedule once per
 * (configuration, dims, block shapes) on the first volumes of the input and
 * captures each (arguments, scratch) combination as a CUDA graph (pinned or
 * device buffers; RFBA_TUNE=0 / RFBA_GRAPH=0 turn either off). No counterpart
 * in the reference. */
int rfba_ctx_last_schedule(rfba_ctx* ctx, int* tile_rows, int* tile_order, int* graph, int* tuned);

/* Text of the last error on the calling thread ("" if none). */
const char* rfba_last_error(void);

/* Library version string. */
const char* rfba_version(void);

#ifdef __cplusplus
}
#endif
#endif /* RFBA_SRRF_H */
