/*
 * gbnufft — C ABI of the GB300 NUFFT library (libgbnufft.so).
 *
 * This is the boundary that replaces the raw-plan layer of mri-nufft
 * (RawFinufftPlan, src/mrinufft/operators/interfaces/finufft.py:23-80, and
 * RawCufinufftPlan, src/mrinufft/operators/interfaces/cufinufft.py:51-137)
 * together with the per-coil Python loops above it
 * (src/mrinufft/operators/base.py:949-1139 and
 * src/mrinufft/operators/interfaces/cufinufft.py:357-1178).
 *
 * Conventions
 *  - every array argument is a device pointer (CUDA global memory) owned by
 *    the caller, complex data is interleaved complex64 (float re, float im),
 *    images are C-ordered with image axis d paired with sample coordinate d;
 *  - sample coordinates are float32 radians in [-pi, pi) (values outside are
 *    folded periodically), one array per image axis;
 *  - type 2 ("op"):  y_j = scale * sum_n x_n exp(isign * i k_j . n)
 *    type 1 ("adj"): x_n = scale * sum_j c_j exp(isign * i k_j . n)
 *    with n in [-floor(N/2), N - floor(N/2)) per axis;
 *  - every call is asynchronous on `stream` except gbn_setpts, which
 *    synchronises `stream` once to size its work table;
 *  - no C++ exception crosses this interface: each call returns a status
 *    code (GBN_OK == 0) and gbn_last_error() describes the last failure of
 *    the calling thread;
 *  - a plan is not thread-safe; concurrent calls on one plan race.
 */
#ifndef GBNUFFT_H
#define GBNUFFT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbn_plan_s* gbn_plan;
/* Layout-compatible with cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* gbn_stream;

#define GBN_OK 0
#define GBN_ERR_ARG 1     /* invalid argument (shape, pointer, size) */
#define GBN_ERR_CUDA 2    /* CUDA runtime error */
#define GBN_ERR_CUFFT 3   /* cuFFT error */
#define GBN_ERR_NOMEM 4   /* device allocation failed */
#define GBN_ERR_STATE 5   /* call out of order (e.g. exec before setpts) */

/* Library version as 10000*major + 100*minor + patch. */
int gbn_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* gbn_last_error(void);

/*
 * Create a plan for `dim`-dimensional (2 or 3) transforms of image shape
 * n_modes[0..dim-1].  Replaces finufft.Plan(2, shape, n_trans, eps, ...)
 * (finufft.py:43-50) and cufinufft Plan(typ, shape, n_trans, eps, ...)
 * (cufinufft.py:83-90).
 *   upsampfac : fine-grid oversampling (2.0 in mri-nufft's default path)
 *   eps       : requested relative accuracy (sets kernel width and shape)
 *   ntrans    : transforms (coils) processed per pass; fine-grid memory is
 *               ntrans * prod(nf) * 8 bytes
 *   spread_only : 1 = only spread / interpolate on a grid of n_modes cells
 *               with no FFT and no deapodisation (finufft's spreadinterponly,
 *               used by the pipe density estimate, finufft.py:225-232)
 *   device    : CUDA device ordinal the plan lives on
 */
int gbn_plan_create(int dim, const int64_t* n_modes, double upsampfac, double eps,
                    int ntrans, int spread_only, int device, gbn_plan* out);

/* Free a plan and its device memory. */
int gbn_plan_destroy(gbn_plan plan);

/* Kernel width, ES beta, fine grid nf[3] and bin sizes bins[3] of a plan
 * (unused axes report 1). Any output pointer may be NULL. */
int gbn_plan_info(gbn_plan plan, int* width, double* beta, int64_t* nf, int* bins);

/* Device bytes currently held by the plan. */
int gbn_plan_device_bytes(gbn_plan plan, int64_t* bytes);

/*
 * Tune a plan (no counterpart in the reference; used by the autotuner):
 *   bins          spatial bin extent per axis in fine cells (NULL: keep)
 *   interp_method 0 shared-memory tiles, 1 direct from the fine grid,
 *                 3 double-buffered tiles, 4 warp-cooperative direct,
 *                 5 tiles + warp-cooperative (3D); -1 keeps the current one
 *   maxsub_cap    largest subproblem (samples per CTA); 0 keeps it
 * Changing bins or maxsub_cap invalidates the points: call gbn_setpts again.
 */
int gbn_plan_tune(gbn_plan plan, const int* bins, int interp_method, int maxsub_cap);

/*
 * Set the non-uniform points: M samples, one float32 device array per image
 * axis (k2 ignored in 2D).  Bin-sorts the points on the device.  Replaces
 * Plan.setpts (finufft.py:55-62, cufinufft.py:94-113).
 */
int gbn_setpts(gbn_plan plan, int64_t M, const float* k0, const float* k1, const float* k2,
               gbn_stream stream);

/*
 * Forward operator (type 2) for n_batchs x n_coils transforms, replacing
 * FourierOperatorSimple.op/_op_sense/_op_calibless (base.py:949-1010) and
 * MRICufiNUFFT._op_sense_device/_op_calibless_device (cufinufft.py:478-500,
 * 609-620):
 *   smaps != NULL (SENSE):  img (B, *N), smaps (C, *N), ksp (B, C, M),
 *                            ksp[b, c] = scale * F(smaps[c] * img[b])
 *   smaps == NULL:           img (B, C, *N), ksp (B, C, M)
 * isign is -1 for mri-nufft's op and +1 for its trajectory-gradient plan.
 */
int gbn_op(gbn_plan plan, const void* img, const void* smaps, void* ksp, int n_batchs,
           int n_coils, float scale, int isign, gbn_stream stream);

/*
 * Adjoint operator (type 1), replacing FourierOperatorSimple.adj_op /
 * _adj_op_sense / _adj_op_calibless / _adj_op (base.py:1015-1073) and
 * MRICufiNUFFT._adj_op_sense_device / _adj_op_calibless_device with the
 * coil-combine kernel (cufinufft.py:743-770, gpu_utils.py:12-24):
 *   density (M floats) may be NULL; it multiplies the k-space data;
 *   smaps != NULL: ksp (B, C, M) -> img (B, *N) = scale * sum_c conj(smaps[c]) F^H(d ksp[b,c])
 *   smaps == NULL: ksp (B, C, M) -> img (B, C, *N)
 */
int gbn_adj(gbn_plan plan, const void* ksp, const float* density, const void* smaps, void* img,
            int n_batchs, int n_coils, float scale, int isign, gbn_stream stream);

/*
 * Data-consistency gradient A^H (A x - y), replacing
 * FourierOperatorSimple.data_consistency / _grad_sense / _grad_calibless
 * (base.py:1075-1139) and MRICufiNUFFT._dc_sense_device /
 * _dc_calibless_device (cufinufft.py:1084-1178):
 *   grad = scale * sum_c conj(s_c) F^H(d * (scale * F(s_c x) - y_c))
 * with the same SENSE / calibrationless layouts as gbn_op / gbn_adj.
 */
int gbn_dc(gbn_plan plan, const void* img, const void* obs, const float* density,
           const void* smaps, void* grad, int n_batchs, int n_coils, float scale,
           gbn_stream stream);

/*
 * Pipe density iterations on a spread_only plan (one transform): `iters`
 * times w <- w / |scale2 * interp(spread(w))|, with w complex64 of length M.
 * Replaces the loop of MRIfinufft.pipe / MRICufiNUFFT.pipe
 * (finufft.py:233-239, cufinufft.py:1319-1325).
 */
int gbn_pipe(gbn_plan plan, void* w, int iters, float scale2, gbn_stream stream);

/*
 * Trajectory gradient of the forward operator, replacing
 * _backward_op_samples (operators/autodiff.py:22-41):
 *   grad[j, d] = sum_{b,c} Re(conj(dy[b,c,j]) d/dk_{j,d} op(img)[b,c,j])
 * evaluated with the derivative of the spreading kernel.  grad is (M, dim)
 * float32 and is overwritten.  Layouts as gbn_op; dy as ksp.
 */
int gbn_grad_traj_op(gbn_plan plan, const void* img, const void* smaps, const void* dy,
                     float* grad, int n_batchs, int n_coils, float scale, gbn_stream stream);

/*
 * Trajectory gradient of the adjoint operator, replacing
 * _backward_adj_samples (operators/autodiff.py:69-86):
 *   grad[j, d] = sum_{b,c} Re(y[b,c,j] d/dk_{j,d} op_+(conj(dx))[b,c,j])
 * where op_+ is the isign=+1 forward operator with conjugated coil maps.
 * dx has the image layout of gbn_op, y the k-space layout.
 */
int gbn_grad_traj_adj(gbn_plan plan, const void* dx, const void* smaps, const void* y,
                      float* grad, int n_batchs, int n_coils, float scale, gbn_stream stream);

/*
 * Batches: many independent plans (uneven image size, sample count and coil
 * count, same dim and kernel width) executed together.  No counterpart in the
 * reference, whose only batching is n_trans chunks of one trajectory
 * (base.py:904-914, cufinufft.py:259-269).  Each stage of a batched op / adj
 * is ONE persistent launch of this library over a work table covering every
 * instance (pad, interp; zero, spread, crop), plus one cuFFT call per
 * instance.  Every plan needs gbn_setpts and ntrans >= its coil count.
 * gbn_batch_bind fixes the device buffers of every instance (image, coil maps
 * or NULL, k-space, density or NULL, scale, coil count) so that
 * gbn_batch_op / gbn_batch_adj take only a stream and can be captured in a
 * CUDA graph:
 *   op:  ksp_i = scale_i F(smaps_i img_i)      (calibrationless: F(img_i))
 *   adj: img_i = scale_i sum_c conj(smaps_ic) F^H(d_i ksp_ic)
 */
typedef struct gbn_batch_s* gbn_batch;
int gbn_batch_create(int n, const gbn_plan* plans, gbn_batch* out);
int gbn_batch_bind(gbn_batch batch, void* const* imgs, const void* const* smaps, void* const* ksps,
                   const float* const* densities, const float* scales, const int* n_coils);
int gbn_batch_op(gbn_batch batch, gbn_stream stream);
int gbn_batch_adj(gbn_batch batch, gbn_stream stream);
int gbn_batch_destroy(gbn_batch batch);

/*
 * Toeplitz embedding of the Gram operator A^H W A (toeplitz.py:35-96
 * compute_toeplitz_kernel, 193-269 apply_toeplitz_kernel; base.py:315-363
 * gram_op with toeplitz=True).  A^H W A x is the linear convolution of x
 * with psf(m) = sum_j w_j exp(+i k_j . m), |m_d| < N_d, i.e. a circular
 * convolution on a grid of nf_d >= 2 N_d - 1 cells per axis.
 *
 *   gbn_toep_create: psf = type-1 transform of the weights (null: ones) on
 *     2N modes (a temporary plan sharing the trajectory k0..k2 of `plan`),
 *     placed at lag m -> m mod nf on the circulant grid (nf = the smallest
 *     even 2-3-5-smooth size >= 2N), then kernel K = Re(FFT(psf)) (real for
 *     real weights).  The handle owns K and fine grids for plan's ntrans.
 *   gbn_toep_apply: per coil pass, zero-pad (x * s_c) into the circulant
 *     grid, FFT, multiply by K, inverse FFT, crop with conj(s_c) coil sum
 *     (smaps null: calibrationless, one image per coil), times
 *     scale / prod(nf).  A^H W A x = apply(x) with scale 1 (times the
 *     operator's 1/norm^2).
 *   gbn_toep_info: nf per axis (unused axes 1);  gbn_toep_kernel: copies K
 *     (prod(nf) floats, C order) into `dst` (device).
 * The reference builds the same kernel from 2^(d-1) modulated adjoints on
 * the N grid and keeps its real spectrum on the 2N grid; where nf = 2N the
 * two kernels hold the same values.
 */
typedef struct gbn_toep_s* gbn_toep;
int gbn_toep_create(gbn_plan plan, int64_t M, const float* k0, const float* k1, const float* k2,
                    const float* weights, gbn_toep* out, gbn_stream stream);
int gbn_toep_info(gbn_toep toep, int64_t* nf);
int gbn_toep_kernel(gbn_toep toep, float* dst, gbn_stream stream);
int gbn_toep_apply(gbn_toep toep, const void* img, const void* smaps, void* out, int B, int C,
                   float scale, gbn_stream stream);
int gbn_toep_destroy(gbn_toep toep);
/* The handle's circulant-grid plan (owned by the handle), for gbn_profile /
 * gbn_profile_read of its pad / FFT / multiply / crop stages. */
int gbn_toep_plan(gbn_toep toep, gbn_plan* out);

/*
 * Served-solver steps on the Toeplitz Gram, one call per iteration (no
 * reference counterpart as single calls; they fuse the loop bodies of
 * extras/optim.py:859-893 and base.py:1196-1212 for device-resident state):
 *   gbn_toep_cg_iter: grad_new = A^H A image - rhs (rhs = A^H y, the same
 *     image layout; scale = 1/norm^2), then the dots of gbn_cg_update's
 *     state[0..6] and the update of gbn_cg_update.
 *   gbn_toep_power_iter: x_new = A^H W A x (one image, no maps), then
 *     state[0] = |x_new|^2 and the step of gbn_power_step.
 */
int gbn_toep_cg_iter(gbn_toep toep, void* image, const void* smaps, const void* rhs, void* grad,
                     void* grad_new, void* velocity, double* state, const float* lipschitz, int B,
                     int C, float scale, float tol, gbn_stream stream);
int gbn_toep_power_iter(gbn_toep toep, void* x, void* x_new, double* state, float* lipschitz,
                        float scale, gbn_stream stream);

/*
 * Stacked NUFFT z-axis passes (stacked.py:36-330, MRIStackedNUFFT: 2D
 * trajectory repeated on the z_index planes of a 3D image, last axis
 * Cartesian).  gbn_stack_fwd: for C coils, per coil s_c * x (SENSE: `img` is
 * one nx x ny x nz image and `smaps` C maps; calibless: `img` holds C
 * images, smaps null), the centred orthonormal DFT along z divided by
 * sqrt(2) (fftshift(fft(ifftshift(.), norm="ortho")) / sqrt(2),
 * stacked.py:178-194), and the kept planes written as C * n_index images of
 * nx x ny (coil major) for a 2D NUFFT of C * n_index transforms.
 * gbn_stack_adj: the adjoint (planes back into a zero stack, inverse
 * centred DFT / sqrt(2), coil combine with conj(smaps), or one image per
 * coil), added to `img` when `accumulate`.
 */
typedef struct gbn_stack_s* gbn_stack;
int gbn_stack_create(const int64_t* shape, const int* z_index, int n_index, int device,
                     gbn_stack* out);
int gbn_stack_fwd(gbn_stack stack, const void* img, const void* smaps, void* out, int C,
                  gbn_stream stream);
int gbn_stack_adj(gbn_stack stack, const void* in, const void* smaps, void* img, int C,
                  int accumulate, gbn_stream stream);
int gbn_stack_destroy(gbn_stack stack);

/*
 * Off-resonance correction (off_resonance.py:233-338, MRIFourierCorrected):
 * y = sum_l B_l * A(C_l x) with time interpolators B (NK x L, complex64,
 * row-major; sample j of a shot uses row j mod NK) and spatial interpolators
 * C_l.  The L interpolators run as L * C transforms of one gbn_op / gbn_adj
 * call whose coil maps are the products C_l s_c; these two passes combine
 * them:
 *   gbn_orc_reduce: y[b][c][j] = sum_l B[j][l] yl[b][l C + c][j]
 *   gbn_orc_expand: yl[b][l C + c][j] = conj(B[j][l]) y[b][c][j]
 * for nb batch items, C coils and M samples (a multiple of NK).
 */
int gbn_orc_reduce(const void* yl, const void* B, void* y, int nb, int L, int C, int64_t M,
                   int64_t NK, gbn_stream stream);
int gbn_orc_expand(const void* y, const void* B, void* yl, int nb, int L, int C, int64_t M,
                   int64_t NK, gbn_stream stream);

/*
 * Stage timing.  gbn_profile(plan, 1) clears the counters and records a pair
 * of CUDA events on the launch stream around every launch of a stage;
 * gbn_profile(plan, 0) stops recording.  gbn_profile_read waits for the
 * recorded events and returns the summed device time and number of launches
 * of one stage (GBN_STAGE_*), or with stage = -1 the time of all stages and
 * the number of kernels this library launched through the plan since the
 * last gbn_profile call.  No counterpart in the reference (which times
 * nothing); it feeds the roofline figures of the benchmark.
 */
#define GBN_STAGE_PAD 0
#define GBN_STAGE_FFT 1
#define GBN_STAGE_INTERP 2
#define GBN_STAGE_SPREAD 3
#define GBN_STAGE_CROP 4
#define GBN_STAGE_ZERO 5
#define GBN_STAGE_GRAD 6
#define GBN_STAGE_KMUL 7
#define GBN_STAGES 8
int gbn_profile(gbn_plan plan, int enable);
int gbn_profile_read(gbn_plan plan, int stage, double* total_ms, int64_t* count);

/*
 * FP64-accumulated reductions on complex64 vectors, used by the CG solver
 * and the power method (extras/optim.py:872-878, base.py:1200-1206):
 *   gbn_norm2_f64: out[0] = sum |x_i|^2
 *   gbn_dotu_f64:  out[0] + i out[1] = sum a_i b_i  (conj_a: sum conj(a_i) b_i)
 * `out` is a device pointer to doubles.
 */
int gbn_norm2_f64(const void* x, int64_t n, double* out, gbn_stream stream);
int gbn_dotu_f64(const void* a, const void* b, int64_t n, int conj_a, double* out,
                 gbn_stream stream);

/*
 * Device-side solver steps, so that a whole CG reconstruction runs without a
 * host synchronisation (the served form keeps many solves in flight).
 *
 * gbn_cg_update: one Polak-Ribiere step of extras/optim.py:866-881 on complex64
 *   vectors of length n.  state (doubles, device) holds [0,1] dot(g_new, g_new),
 *   [2,3] dot(g_new, g), [4,5] dot(g, g) (numpy's non-conjugating dot, as from
 *   gbn_dotu_f64), [6] |g_new|^2 (gbn_norm2_f64), [7] done flag.  Unless done
 *   or |g_new| <= tol (then done is set, the reference's early exit):
 *   beta = max(0, (dot(g_new,g_new) - dot(g_new,g)) / dot(g,g)) under numpy's
 *   complex ordering,
 *   velocity = g_new + beta velocity, image -= velocity / L, grad = g_new.
 *   lipschitz is a device float.
 * gbn_power_step: the normalisation of one power-method iteration
 *   (operators/base.py:1202-1209): state [0] |x_new|^2, [1] previous norm,
 *   [2] current estimate, [3] converged flag; x = x_new / |x_new| and the
 *   estimate goes to *lipschitz, until |previous - current| < 1e-6.
 * gbn_scale_ratio: x *= sqrt(num2 / den2) with both squared norms on the
 *   device (the scaling of _scaled_dcp, extras/optim.py:151-165).
 */
int gbn_cg_update(int64_t n, const void* grad_new, void* grad, void* velocity, void* image,
                  double* state, const float* lipschitz, float tol, gbn_stream stream);
int gbn_power_step(int64_t n, const void* x_new, void* x, double* state, float* lipschitz,
                   gbn_stream stream);
int gbn_scale_ratio(int64_t n, void* x, const double* num2, const double* den2, gbn_stream stream);

/*
 * Pipe density iterations that allocate nothing.  No counterpart in the
 * reference: it is the gbn_pipe iteration for callers that cannot allocate
 * device memory at the time they need it (a process whose device memory is
 * held by a framework's pool, or a real-time reconstruction service that
 * forbids allocation after start-up).  It needs no plan: the image-size grid
 * lives in a fixed device array of GBN_STATIC_GRID_CELLS complex64 cells
 * (16 MiB, held on every GPU that loads the library until exit), and the
 * samples are used unsorted.  Same arguments and result as
 * gbn_plan_create(dim, n_modes, osf, eps, 1, 1, dev) + gbn_setpts + gbn_pipe:
 * `iters` times w <- w / |scale2 * interp(spread(w))| on the n_modes grid,
 * w complex64 of length M, coordinates float32 radians, on the current
 * device; osf <= 1 takes the osf = 2 kernel, as gbn_plan_create does.
 * Grids of more than GBN_STATIC_GRID_CELLS cells are rejected (GBN_ERR_ARG)
 * before anything runs.  Every call looks the array's device address up with
 * cudaGetSymbolAddress (no allocation); the first call on a device also
 * loads the module there and should come before any stream capture.  Every
 * call shares the array (each iteration clears it first): calls whose work
 * overlaps on the GPU race and must be serialised by the caller.
 */
#define GBN_STATIC_GRID_CELLS (1 << 21)
int gbn_pipe_static(int dim, const int64_t* n_modes, double osf, double eps, int64_t M,
                    const float* k0, const float* k1, const float* k2, void* w, int iters,
                    float scale2, gbn_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* GBNUFFT_H */
