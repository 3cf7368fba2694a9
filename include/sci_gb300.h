/*
 * sci_gb300.h -- C ABI of the GB300-native GAP-TV / ADMM-TV library
 * (libsci_gb300.so, built from sci-algorithms_gb300/csrc for sm_103a).
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer to float32 data in the planar
 *     layout B x H x W (frame-major, W fastest) unless stated otherwise.
 *     The reference keeps frames last (H x W x B, numpy C order,
 *     PnP_SCI/python/utils.py:15,26); callers convert once at the boundary.
 *   - 2-D maps (measurement y, Phi_sum, y1) are H x W.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  All work is
 *     stream-ordered; no call synchronises the device unless stated.
 *   - Ownership: the caller allocates every buffer, including the workspace
 *     whose size the *_workspace_bytes queries return.  The library keeps
 *     no device memory of its own apart from cached CUDA graphs.
 *   - Errors: every function returns SCI_OK (0) or a negative SCI_ERR_*
 *     code; sci_last_error() returns the message of the last failure on the
 *     calling thread.  No kernel traps; device-side waits are bounded.
 *   - Inputs are never modified unless the argument is documented in/out.
 */
#ifndef SCI_GB300_H
#define SCI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCI_OK 0
#define SCI_ERR_INVALID_ARG -1
#define SCI_ERR_CUDA -2
#define SCI_ERR_UNSUPPORTED -3
#define SCI_ERR_WORKSPACE -4
#define SCI_ERR_TIMEOUT -5

/* Library version (major*10000 + minor*100 + patch). */
int sci_version(void);

/* Copies the last error message of this thread into buf (NUL-terminated,
 * truncated to n bytes).  Returns the full message length. */
int sci_last_error(char *buf, size_t n);

/* Reads the device status word into *status and, with clear != 0, resets
 * it.  Bit 0 is set when a bounded device-side wait of a bulk-copy kernel
 * (the GAP projection of sci_proj_gap with a packed mask, the batched and
 * convolution kernels) gave up; bit 1 when a wait of the batched solve's
 * work queue (sci_batch_gap_tv) gave up.  The results of such a launch are
 * not valid.  Synchronous.  No counterpart in the reference (library
 * plumbing). */
int sci_device_status(unsigned int *status, int clear);

/* Exercises the error path of the bounded device-side waits: one block
 * waits, `polls` times at most (1 .. 2^20), on a barrier that expects bytes
 * no copy delivers, then sets bit 0 of the device status word and returns.
 * For tests of that path; the context stays usable.  No counterpart in the
 * reference. */
int sci_selftest_bounded_wait(unsigned int polls, void *stream);

/* ---------------------------------------------------------- L1 operators */

/* y = sum_b phi_b .* x_b.
 * Replaces A_(x, Phi)            PnP_SCI/python/utils.py:10-15 */
int sci_A(const float *x, const float *phi, float *y,
          int64_t B, int64_t H, int64_t W, void *stream);

/* x_b = phi_b .* y.
 * Replaces At_(y, Phi)           PnP_SCI/python/utils.py:17-26 */
int sci_At(const float *y, const float *phi, float *x,
           int64_t B, int64_t H, int64_t W, void *stream);

/* phisum = sum_b phi_b, entries equal to 0 replaced by 1 when guard_zero.
 * Replaces the mask_sum lines    PnP_SCI/python/pnp_sci_algo.py:491-492 */
int sci_phisum(const float *phi, float *phisum, int64_t B, int64_t H,
               int64_t W, int guard_zero, void *stream);

/* Packs a binary mask (every entry exactly 0 or 1) into one uint32 word per
 * pixel, bit b = phi_b (B <= 32).  Returns SCI_ERR_INVALID_ARG through
 * *nonbinary_flag (device int, set to 1) if an entry is neither 0 nor 1;
 * the caller must then use the float mask.  No reference counterpart: a
 * storage format for binary coded apertures (pnp_sci_test_orig.py:135-137
 * masks are 0/1 after normalisation). */
int sci_pack_mask(const float *phi, uint32_t *bits, int *nonbinary_flag,
                  int64_t B, int64_t H, int64_t W, void *stream);

/* ------------------------------------------------ projections (fused K1) */

/* One GAP projection over the B-frame stack in a single pass:
 *   yb = A(x); accelerate: y1 += y - yb, r = (y1 - yb)/phisum;
 *   else r = (y - yb)/phisum;   x_out = x + lambda * At(r).
 * y1 is in/out (ignored when accelerate == 0).  mask_bits (nullable) is
 * the packed form of phi; when given, phi may be NULL.
 * Replaces pnp_sci_algo.py:640-645 (gap_denoise, GAP and GAP_acc). */
int sci_proj_gap(const float *x, const float *phi, const uint32_t *mask_bits,
                 const float *y, float *y1, const float *phisum, float *x_out,
                 float lambda, int accelerate,
                 int64_t B, int64_t H, int64_t W, void *stream);

/* Residual map of one GAP projection, without writing the projected stack:
 *   yb = A(x); accelerate: y1 += y - yb, c = (y1 - yb)/phisum;
 *   else c = (y - yb)/phisum.            (c, y1: H x W; y1 in/out)
 * The update x + lambda At(c) is then applied by the TV kernel while it
 * reads x (the fused GAP-TV iteration).  Needs H*W % 4 == 0 and 16-byte
 * aligned buffers.  Replaces the first half of pnp_sci_algo.py:640-645. */
int sci_gap_residual(const float *x, const float *phi, const uint32_t *mask_bits,
                     const float *y, float *y1, const float *phisum, float *c,
                     int accelerate, int64_t B, int64_t H, int64_t W, void *stream);

/* One ADMM projection:  t = theta + b; yb = A(t);
 *   x = t + lambda * At((y - yb)/(phisum + gamma));  v = x - b.
 * Writes v (the TV input) and, when x_out is non-NULL, x.
 * Replaces pnp_sci_algo.py:808-809 (admm_denoise) and the x - b of :812. */
int sci_proj_admm(const float *theta, const float *b, const float *phi,
                  const uint32_t *mask_bits, const float *y,
                  const float *phisum, float *v, float *x_out, float lambda,
                  float gamma, int64_t B, int64_t H, int64_t W, void *stream);

/* ------------------------------------------------------ Chambolle TV (K2) */

/* Bytes of device workspace sci_tv_chambolle needs for these sizes. */
int sci_tv_workspace_bytes(int64_t nframes, int64_t H, int64_t W,
                           int n_iter_max, size_t *bytes);

/* Per-frame Chambolle TV (scikit-image 0.16 denoise_tv_chambolle
 * semantics, including its energy stop test with eps) of nframes H x W
 * frames: u = TV(f).  resid (nullable) receives u - f (the ADMM multiplier
 * update b = theta - v).  steps (nullable, device int[nframes]) receives
 * the number of executed Chambolle steps per frame.  energy (nullable,
 * device double[nframes * n_iter_max * 2]) receives, for every step k the
 * stop test evaluates, H*W*E_k = sum (div p_k)^2 + weight * sum |grad u_k|
 * in energy[(f*n_iter_max + k)*2] (the odd entries stay 0).
 * Replaces denoise_tv_chambolle(x, weight, n_iter_max, multichannel=True)
 * as called at PnP_SCI/python/pnp_sci_algo.py:650 and :812-813. */
int sci_tv_chambolle(const float *f, float *u, float *resid, int64_t nframes,
                     int64_t H, int64_t W, float weight, float eps,
                     int n_iter_max, int *steps, double *energy,
                     void *workspace, size_t workspace_bytes, void *stream);

/* Allocation-free variant of sci_tv_chambolle, for callers that cannot
 * allocate device memory (a host framework that owns all device memory
 * through its own pool, a plug-in handed only its input and output
 * buffers, a loop where cudaMalloc would synchronise the device).  Its
 * scratch is a fixed 64 KiB array in the library's device image (kept on
 * every GPU that loads the library until exit), so it needs no workspace
 * argument.  Limits: n_iter_max <= 5 and nframes * n_iter_max * 16 bytes
 * (+ 8 bytes per frame, with alignment) <= 64 KiB (nframes <= 742 at
 * n_iter_max = 5);
 * larger requests return SCI_ERR_INVALID_ARG.  All calls share the array:
 * calls whose work overlaps on the GPU race and must be ordered by the
 * caller.  The first call on a device looks up the array's address; make
 * it before any stream capture on that device.  No counterpart in the
 * reference (which allocates on the host through numpy). */
int sci_tv_chambolle_noalloc(const float *f, float *u, float *resid,
                             int64_t nframes, int64_t H, int64_t W,
                             float weight, float eps, int n_iter_max,
                             int *steps, void *stream);

/* ------------------------------------- MATLAB-twin TV denoisers (next row) */

/* The denoisers the MATLAB GAP loop selects with its tvm switch
 * (PnP_SCI/matlab/algorithms/gapdenoise.m:92-112), by kind: */
#define SCI_TVM_ATV_CLIPA 1   /* TV_denoising.m(v, lambda, iters)          */
#define SCI_TVM_ATV_CLIPB 2   /* TV_denoising_clip_LB.m                    */
#define SCI_TVM_ATV_CHAM 3    /* tvdenoise_cham_ATV2D.m                    */
#define SCI_TVM_ATV_FGP 4     /* fgp_denoise_ATV2D.m                       */
#define SCI_TVM_ITV2D_CHAM 5  /* tvdenoise_cham_ITV2D.m                    */
#define SCI_TVM_ITV2D_FGP 6   /* fgp_denoise_ITV2D.m                       */
#define SCI_TVM_ITV3D_CHAM 7  /* tvdenoise_cham_ITV3D.m (norm over frames) */
#define SCI_TVM_ITV3D_FGP 8   /* fgp_denoise_ITV3D.m (norm over frames)    */

/* Bytes of device workspace sci_tv_matlab needs for up to `iters`
 * iterations. */
int sci_tv_matlab_workspace_bytes(int kind, int64_t nframes, int64_t H,
                                  int64_t W, int iters, size_t *bytes);

/* u = denoiser `kind`(f, lambda, iters) on the planar stack of nframes
 * H x W frames (H, W >= 2), with the file's own parameter: lambda is the
 * clip bound / ROF weight of TV_denoising*.m and fgp_denoise_*.m, and the
 * fidelity weight of tvdenoise_cham_*.m (gapdenoise.m passes tvweight and
 * 1/tvweight respectively; 5 iterations, 2 for the FGP files).  A
 * one-frame stack takes MATLAB's 2-D branch of the file.
 * Replaces the calls at gapdenoise.m:94-108. */
int sci_tv_matlab(int kind, const float *f, float *u, int64_t nframes,
                  int64_t H, int64_t W, float lambda, int iters,
                  void *workspace, size_t workspace_bytes, void *stream);

/* -------------------------------------------------- metrics (diagnostics) */

/* out[0] += sum_i (a_i - b_i)^2 in float64 (PSNR numerator for
 * psnr()/compare_psnr, PnP_SCI/python/utils.py:28-36). */
int sci_sqerr_accum(const float *a, const float *b, int64_t n, double *out,
                    void *stream);

/* ------------------------------------------------------ solvers (L2 loop) */

/* Options shared by the solvers. */
typedef struct sci_solve_opts {
    int iters;               /* total GAP/ADMM iterations                   */
    const float *lambdas;    /* HOST array [iters]: lambda_k                */
    const float *weights;    /* HOST array [iters]: tv_weight_k             */
    int tv_iter_max;         /* Chambolle steps per TV call (n_iter_max)    */
    float eps;               /* TV stop tolerance (scikit-image eps)        */
    int accelerate;          /* GAP: 1 = GAP_acc                            */
    float gamma;             /* ADMM: gamma                                 */
    const float *gammas;     /* nullable HOST array [iters]: gamma_k        */
    const float *orig;       /* nullable: ground truth for PSNR per iter    */
    double *sqerr;           /* nullable device double[iters]: sum sq. err. */
    int *tv_steps;           /* nullable device int[iters * B]              */
    int use_graph;           /* 1: capture the loop in a CUDA graph (cached) */
    int tvm;                 /* 0: scikit-image Chambolle (tv_iter_max steps,
                              * stop test eps); SCI_TVM_*: that MATLAB
                              * denoiser with tv_iter_max iterations and
                              * weights as gapdenoise.m's tvweight           */
    double *resid_norm;      /* nullable device double[iters]: ||r_k||^2 of
                              * iteration k's projection residual, summed in
                              * FP64 by the projection kernel: r = (y1 - A x)
                              * / Phi_sum for GAP_acc, (y - A x) / Phi_sum for
                              * GAP (pnp_sci_algo.py:640-645), (y - A(theta +
                              * b)) / (Phi_sum + gamma) for ADMM (:808-809)  */
} sci_solve_opts;

/* Workspace bytes for sci_gap_tv / sci_admm_tv. */
int sci_solver_workspace_bytes(int64_t B, int64_t H, int64_t W,
                               const sci_solve_opts *opts, size_t *bytes);

/* GAP-TV: x_out = gap_denoise(y, phisum, A, At, x0=x0, ...).x for
 * denoiser='tv' (PnP_SCI/python/pnp_sci_algo.py:536-706).  x0 and x_out may
 * alias.  phi or mask_bits (one may be NULL). */
int sci_gap_tv(const float *y, const float *phi, const uint32_t *mask_bits,
               const float *phisum, const float *x0, float *x_out,
               int64_t B, int64_t H, int64_t W, const sci_solve_opts *opts,
               void *workspace, size_t workspace_bytes, void *stream);

/* ADMM-TV: x_out = admm_denoise(y, phisum, A, At, x0=x0, ...).x
 * (PnP_SCI/python/pnp_sci_algo.py:708-864); returns x, not theta. */
int sci_admm_tv(const float *y, const float *phi, const uint32_t *mask_bits,
                const float *phisum, const float *x0, float *x_out,
                int64_t B, int64_t H, int64_t W, const sci_solve_opts *opts,
                void *workspace, size_t workspace_bytes, void *stream);

/* ------------------------------------------- spectral (CASSI) operators (K3) */
/* Single coded aperture phi (H x W) followed by a dispersion that shifts
 * band b by step*b pixels along W onto an H x Wd detector,
 * Wd = W + step*(L-1).  No Python counterpart in the reference; the
 * MATLAB CASSI test uses the same model with a pre-shifted mask and
 * Phisum = sum(mask.^2, 3) (DeSCI/test_desci_cassi.m:58-62). */

/* y[h, w + step b] += phi[h, w] x_b[h, w]   (x: L x H x W, y: H x Wd) */
int sci_cassi_A(const float *x, const float *phi, float *y, int64_t L,
                int64_t H, int64_t W, int step, void *stream);

/* x_b[h, w] = phi[h, w] y[h, w + step b]    (the transposed unshift) */
int sci_cassi_At(const float *y, const float *phi, float *x, int64_t L,
                 int64_t H, int64_t W, int step, void *stream);

/* phisum[h, w'] = sum_b phi[h, w' - step b]^2, zeros -> 1 when guard_zero */
int sci_cassi_phisum(const float *phi, float *phisum, int64_t L, int64_t H,
                     int64_t W, int step, int guard_zero, void *stream);

int sci_cassi_workspace_bytes(int64_t L, int64_t H, int64_t W, int step,
                              int tv_iter_max, size_t *bytes);

/* GAP-TV with the CASSI operators (gap_denoise, pnp_sci_algo.py:536-706,
 * with A/At = the operators above; per-band Chambolle TV).  Uses
 * opts->iters, lambdas, weights, tv_iter_max, eps, accelerate, orig,
 * sqerr, tv_steps and use_graph (the loop captured once into a cached CUDA
 * graph, as sci_gap_tv does). */
int sci_cassi_gap_tv(const float *y, const float *phi, const float *phisum,
                     const float *x0, float *x_out, int64_t L, int64_t H,
                     int64_t W, int step, const sci_solve_opts *opts,
                     void *workspace, size_t workspace_bytes, void *stream);

/* ------------------------------------- batched uneven GAP-TV (K5) */
/* One measurement of a batch: device pointers (y: H x W, mask_bits: packed
 * binary mask, one uint32 word per pixel, bit b = frame b, B <= 32;
 * phisum: H x W; x: B x H x W, in: x0 (unless init_x0), out: result),
 * sizes (W % 4 == 0, 16-byte aligned buffers), step size, TV weight, and
 * the TV row-chunk height R (0: default; sci_batch_autotune fills it). */
typedef struct sci_batch_item {
    const float *y;
    const uint32_t *mask_bits;
    const float *phisum;
    float *x;
    int64_t B, H, W;
    float lambda;
    float tv_weight;
    int R;
    int cpl;  /* TV columns per lane, 2 or 4 (0: 4; sci_batch_autotune fills it) */
} sci_batch_item;

int sci_batch_workspace_bytes(const sci_batch_item *items, int n, int tv_iter_max,
                              size_t *bytes);

/* Autotuner of the batched solve: times candidate tilings on a few
 * iterations of the batch's own solve (from x0 = At(y / phisum), overwriting
 * every item's x) -- row-chunk heights of 1/2, 1 and 2 times the default for
 * each item's height, and 4 columns per lane for every item or 2 for items
 * at most 256 columns wide -- and writes the fastest into items[i].R and
 * items[i].cpl; with a non-null iters_per_launch it then times 1, 2 or 3
 * iterations per persistent launch against all of them and writes the
 * fastest (0: all in one launch).  Cached per process for the list of
 * shapes.  Synchronises the stream. */
int sci_batch_autotune(sci_batch_item *items, int n, int iters, int tv_iter_max,
                       float eps, int accelerate, int *iters_per_launch,
                       void *workspace, size_t workspace_bytes, void *stream);

/* GAP-TV (pnp_sci_algo.py:536-706, denoiser='tv') of n <= 256 independent
 * measurements, all items advancing together: persistent launches over a
 * device work queue, each running iters_per_launch iterations (0: all) of
 * every item -- per iteration the projection tiles, TV work items and stop
 * tests of all items, a task waiting (bounded) only for earlier tasks of
 * its own item.  With use_graph the whole loop is captured once into a
 * cached CUDA graph.  init_x0: start from At(y / phisum) (else from x).
 * tv_iter_max in [2, 5].  The item table is uploaded synchronously before
 * the work is enqueued.  A wait that gave up sets bit 1 of the device
 * status (sci_device_status). */
int sci_batch_gap_tv(const sci_batch_item *items, int n, int iters,
                     int tv_iter_max, float eps, int accelerate, int init_x0,
                     int use_graph, int iters_per_launch, void *workspace,
                     size_t workspace_bytes, void *stream);

/* Exercises the give-up path of the work queue's bounded waits: one warp
 * waits, `polls` times at most (1 .. 2^20), for a task count that nothing
 * raises, then raises the queue's abort flag, which sets bit 1 of the
 * device status word.  workspace: any device buffer of at least 4 KB (the
 * queue's counters are placed there).  For tests of that path; the context
 * stays usable.  No counterpart in the reference. */
int sci_batch_selftest_queue_wait(unsigned int polls, void *workspace,
                                  size_t workspace_bytes, void *stream);

/* ------------------------------- differentiable unrolled GAP-TV (K4) */
/* A batch of N scenes x_true (N x B x H x W) sharing one learnable mask
 * Phi = sigmoid(logits) (B x H x W) and per-iteration step sizes
 * lambdas (device float[K]):  y = A(x_true), x^0 = At(y / Phi_sum), then K
 * accelerated GAP iterations (pnp_sci_algo.py:641-643) each followed by a
 * fixed tv_iters-step Chambolle TV (no stop test), weight tv_weight;
 * loss = mean (x^K - x_true)^2.  No reference counterpart: the reference's
 * solvers are not differentiable; this is the unrolled form of its
 * gap_denoise loop. */

int sci_unrolled_workspace_bytes(int64_t N, int64_t B, int64_t H, int64_t W,
                                 int K, int tv_iters, size_t *bytes);

/* Forward: writes *loss = sum (x^K - x_true)^2 (device double; divide by
 * N*B*H*W for the mean) and, when x_out is non-NULL, x^K.
 * Keeps the outer iterates in the workspace for sci_unrolled_bwd. */
int sci_unrolled_fwd(const float *logits, const float *lambdas,
                     const float *x_true, int64_t N, int64_t B, int64_t H,
                     int64_t W, int K, int tv_iters, float tv_weight,
                     double *loss, float *x_out, void *workspace,
                     size_t workspace_bytes, void *stream);

/* Reverse pass of the preceding sci_unrolled_fwd on the same workspace and
 * arguments: grad_logits (B x H x W) and grad_lambdas (device double[K])
 * of grad_loss * loss.  Recomputes each TV call from its checkpoint, or,
 * with SCI_UNROLLED_TAPE=1 set for the forward and the workspace query,
 * reads the TV tape the forward kept (when the tapes of all K iterations
 * fit in 48 GiB of workspace; sci_unrolled_workspace_bytes includes them). */
int sci_unrolled_bwd(const float *logits, const float *lambdas,
                     const float *x_true, int64_t N, int64_t B, int64_t H,
                     int64_t W, int K, int tv_iters, float tv_weight,
                     float grad_loss, float *grad_logits, double *grad_lambdas,
                     void *workspace, size_t workspace_bytes, void *stream);

/* ------------------------------------------- CNN denoiser glue (joint/PnP) */
/* Input / output tensors of the FFDNet and FastDVDnet denoisers built from,
 * and turned back into, planar float32 frame stacks (nframes x H x W), so
 * that all frames of a stack go through one batched network call.  The
 * convolutions themselves run in the caller's framework.  Layouts:
 * SCI_CNN_NCHW_F32 planar float32; SCI_CNN_NHWC8_BF16 one 16-byte vector
 * of 8 bfloat16 channels per pixel; SCI_CNN_NHWC8_F32 8 float32 channels
 * per pixel (unused channels 0).  sigma is a device
 * float (the noise level), read at run time so that a captured CUDA graph
 * replays with a new level. */
#define SCI_CNN_NCHW_F32 0
#define SCI_CNN_NHWC8_BF16 1
#define SCI_CNN_NHWC8_F32 2

/* FFDNet input: channel 0 = sigma, channel 1 + 2i + j = pixel (i, j) of
 * each 2 x 2 cell; out is nframes x 5 x ceil(H/2) x ceil(W/2) (NCHW) or
 * nframes x ceil(H/2) x ceil(W/2) x 8 (NHWC8).  Odd sizes repeat the last
 * row / column.  Replaces concatenate_input_noise_map
 * (PnP_SCI/python/packages/ffdnet/functions.py:17-58) as called per frame
 * by ffdnet_vdenoiser (packages/ffdnet/test_ffdnet_ipol.py:133-169). */
int sci_cnn_ffdnet_pack(const float *x, int64_t nframes, int64_t H, int64_t W,
                        const float *sigma, void *out, int layout, void *stream);

/* out = x - depth_to_space(noise), cropped to H x W, clipped to [0, 1] when
 * clip != 0.  noise: nframes x 4 x ceil(H/2) x ceil(W/2) float32 (NCHW) or
 * bfloat16 / float32 NHWC with `channels` (4 or 8) channels per pixel.  Replaces
 * upsamplefeatures (packages/ffdnet/functions.py:60-93) and the
 * subtraction of test_ffdnet_ipol.py:174. */
int sci_cnn_ffdnet_unpack_sub(const float *x, const void *noise, int64_t nframes,
                              int64_t H, int64_t W, int layout, int channels,
                              int clip, float *out, void *stream);

/* FastDVDnet triplet input for the centre frames g = first .. first +
 * count - 1 of src (nframes x Hs x Ws): channels [src[g-1], sigma, src[g],
 * sigma, src[g+1], sigma] (frame indices modulo nframes), reflect-padded at
 * the bottom / right to Hp x Wp (Hp - Hs < Hs, Wp - Ws < Ws).  out: count x
 * 6 x Hp x Wp (NCHW) or count x Hp x Wp x 8 (NHWC8).  Replaces the window gather, padding and
 * noise-map concatenation of fastdvdnet_seqdenoise
 * (packages/fastdvdnet/fastdvdnet.py:117-131) and DenBlock.forward's input
 * (packages/fastdvdnet/models.py:201). */
int sci_cnn_window(const float *src, int64_t nframes, int64_t Hs, int64_t Ws,
                   int64_t Hp, int64_t Wp, int64_t first, int64_t count,
                   const float *sigma, void *out, int layout, void *stream);

/* out[k] = src[first + k] (reflect-padded as in sci_cnn_window) - r[k],
 * k < count, cropped to Ho x Wo, clipped to [0, 1] when clip != 0.  r:
 * count x 1 x Hp x Wp float32 (NCHW) or bfloat16 / float32 NHWC with `channels`
 * channels (channel 0 used).  Replaces DenBlock's `in1 - x` (packages/fastdvdnet/models.py:205)
 * and the crop of fastdvdnet.py:136-140. */
int sci_cnn_center_sub(const float *src, int64_t nframes, int64_t Hs, int64_t Ws,
                       int64_t first, int64_t count, const void *r, int layout,
                       int channels, int64_t Hp, int64_t Wp, int64_t Ho, int64_t Wo,
                       int clip, float *out, void *stream);

/* FastDVDnet's upsampling and skip connection in one pass, bfloat16 NHWC:
 * out[n, 2i+a, 2j+b, c] = a[n, 2i+a, 2j+b, c] + u[n, i, j, (2a+b)*C + c]
 * (a nullable: the shuffle alone).  u is N x h x w x 4C with the
 * upsampling convolution's output channels ordered sub-pixel-major (its
 * channel c*4 + 2a + b moved to (2a+b)*C + c); a, out: N x 2h x 2w x C;
 * C % 8 == 0; 16-byte aligned.  Replaces nn.PixelShuffle(2) of UpBlock
 * and the additions x1 + x2, x0 + x1 of DenBlock.forward
 * (packages/fastdvdnet/models.py:72-84, :202-203). */
int sci_cnn_shuffle_add(const void *a, const void *u, void *out, int64_t N,
                        int64_t h, int64_t w, int64_t C, void *stream);

/* The same on float32 NHWC tensors (C % 4 == 0). */
int sci_cnn_shuffle_add_f32(const float *a, const float *u, float *out, int64_t N,
                            int64_t h, int64_t w, int64_t C, void *stream);

/* 3 x 3 convolution (zero padding 1, stride 1) of a thin input on the
 * tensor cores (tcgen05.mma, float32 accumulation in tensor memory):
 * out[p, n] = act(bias[n] + sum_{tap, c} in[p + tap offset, c] * w[n, tap*8 + c])
 * for every pixel p of nframes x H x W.  in: NHWC8 bfloat16 (8 channels =
 * 16 bytes per pixel, as written by sci_cnn_window / sci_cnn_ffdnet_pack);
 * weights: N x 80 bfloat16 (k = tap*8 + c with tap = 3*dy + dx, k >= 72
 * zero); bias: N float32; out: NHWC bfloat16 with N channels; act = ReLU
 * when relu != 0.  N = 64 or 96.  16-byte aligned buffers.  A timed-out
 * device-side wait sets bit 0 of the status word of sci_device_status.
 * Replaces the first convolution of FastDVDnet's DenBlock (InputCvBlock,
 * packages/fastdvdnet/models.py:29-43, 3 groups of 2 -> 30 channels as
 * one dense 8 -> 96 filter) and of FFDNet (packages/ffdnet/models.py:37-42). */
int sci_cnn_conv_thin(const void *in, const void *weights, const float *bias,
                      void *out, int64_t nframes, int64_t H, int64_t W, int N,
                      int relu, void *stream);

/* FastDVDnet's DenBlock tail in one pass on the tensor cores, bfloat16
 * operands, float32 accumulation:
 *   h = x0 + PixelShuffle(2)(u1), o0 = ReLU(conv3x3(h, w0) + b0) (bfloat16),
 *   e = conv3x3(o0, w1) + b1 (float32), out[k] = src[first + k] - e,
 * src reflect-padded to Hp x Wp as in sci_cnn_center_sub, out cropped to
 * Ho x Wo and clipped to [0, 1] when clip != 0 (count x Ho x Wo float32).
 * x0: count x Hp x Wp x 32 bfloat16 (NHWC); u1: count x Hp/2 x Wp/2 x 128
 * bfloat16 with the upsampling convolution's channels sub-pixel-major (as
 * sci_cnn_shuffle_add); w0: 32 x 288 bfloat16 (k = (3 dy + dx) * 32 + c),
 * b0: 32 float32; w1: 288 bfloat16 (the one output filter), b1: one
 * float32 or NULL (zero).  Both convolutions zero-pad by 1.  Hp, Wp even.
 * A timed-out device-side wait sets bit 0 of the status word of
 * sci_device_status.  Replaces DenBlock.forward's x0 + x1, OutputCvBlock
 * and in1 - x (packages/fastdvdnet/models.py:86-100, :203-205) and the
 * crop of fastdvdnet.py:136-140. */
int sci_cnn_den_tail(const void *x0, const void *u1, const void *w0, const float *b0,
                     const void *w1, const float *b1, const float *src, int64_t nframes,
                     int64_t Hs, int64_t Ws, int64_t first, int64_t count, int64_t Hp,
                     int64_t Wp, int64_t Ho, int64_t Wo, int clip, float *out, void *stream);

/* Per-frame image-quality sums of x against orig (planar nframes x H x W,
 * H, W >= 7): sqerr[f] = sum (orig - x)^2 over frame f, and ssim_sum[f] =
 * the sum of the SSIM map (7 x 7 uniform windows, sample covariance, K1 =
 * 0.01, K2 = 0.03, dynamic range data_range) over the frame cropped by 3
 * pixels, i.e. SSIM = ssim_sum / ((H - 6)(W - 6)) and PSNR =
 * 10 log10(data_range^2 / (sqerr / (H W))).  Device doubles, overwritten.
 * Replaces compare_psnr / compare_ssim(..., data_range=1.) per frame
 * (PnP_SCI/python/pnp_sci_algo.py:702-705, scikit-image 0.16). */
int sci_frame_metrics(const float *orig, const float *x, int64_t nframes,
                      int64_t H, int64_t W, double data_range, double *sqerr,
                      double *ssim_sum, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SCI_GB300_H */
