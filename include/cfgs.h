/*
 * cfgs.h — C ABI of the GB300 (sm_103a) differentiable Gaussian rasteriser.
 *
 * This library is a drop-in for the native half of the `diff_gaussian_rasterization`
 * package that CF-3DGS calls at
 *   scene/gaussian_model_cf.py:811-882   (CF3DGS_Render.render)
 *   gaussian_renderer/__init__.py:38-96  (render)
 *   scene/gaussian_model.py:915-980      (GS_Render.render)
 * The upstream native module (`diff_gaussian_rasterization._C`, un-vendored in the
 * reference tree, .gitmodules:4-6) exposes `rasterize_gaussians`,
 * `rasterize_gaussians_backward` and `mark_visible`; the entry points below replace
 * those three and add the pose-gradient kernels of the CF-3DGS pose solve
 * (scene/gaussian_model_cf.py:123-133, trainer/cf3dgs_trainer.py:261-285).
 *
 * Conventions
 *  - Every pointer is a DEVICE pointer unless its comment says "host".
 *  - The caller owns every buffer. The library allocates nothing and frees nothing;
 *    the *_bytes() functions size the workspaces.
 *  - `stream` is a cudaStream_t (0 = legacy default stream). All work is enqueued on
 *    it; no entry point synchronises unless CfgsSettings.debug is set, except
 *    cfgs_read_counts(), whose job is to read a device value back.
 *  - Every entry point returns a CfgsStatus; nonzero means nothing useful was written.
 *  - Matrices are the 4x4 float tensors CF-3DGS stores on its Camera
 *    (scene/cameras.py:57-74): row-major storage of the TRANSPOSED matrix, i.e. a
 *    point p maps to [p,1] @ M (row-vector convention).
 */
#ifndef CFGS_H
#define CFGS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum CfgsStatus {
  CFGS_OK = 0,
  CFGS_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad SH degree ...            */
  CFGS_ERR_CAPACITY = 2,         /* more tile instances than the binning capacity        */
  CFGS_ERR_LAUNCH = 3,           /* a CUDA launch or runtime call failed                 */
  CFGS_ERR_DEVICE_FLAG = 4,      /* a kernel raised a flag (see CfgsCounts.flags)        */
  CFGS_ERR_TOO_LARGE = 5         /* a size above a documented maximum                    */
} CfgsStatus;

/* Bits of CfgsCounts.flags (raised by kernels, read back with cfgs_read_counts). */
#define CFGS_FLAG_FRUSTUM_VIOLATION 0x1u /* prefiltered=1 but a point was at view z <= 0.2 */
#define CFGS_FLAG_CAPACITY_OVERFLOW 0x2u /* K > binning capacity; outputs are invalid      */
#define CFGS_FLAG_COPY_TIMEOUT 0x4u      /* a bounded wait for an on-chip copy ran out;   */
                                         /* that call's outputs are invalid               */
#define CFGS_FLAG_BARRIER_TIMEOUT 0x8u   /* a bounded grid-wide wait of the one-launch    */
                                         /* binning ran out; outputs are invalid          */

/* Tile size of the screen-space binning (pixels). */
#define CFGS_TILE_X 16
#define CFGS_TILE_Y 16

/* ---- render schedule -----------------------------------------------------------------
 * Launch shape of the two per-tile render kernels, chosen per call (a field of
 * CfgsSettings and of CfgsBatchArgs; the library keeps no schedule of its own). Every
 * schedule gives bit-identical results (each pixel sees the same instances in the same
 * order with the same arithmetic, and each instance's gradient record is summed the same
 * way), so the choice is a pure performance one; cfgs/autotune.py picks it by timing.
 *   fwd_batch: instances staged per round in the forward: 64, 128 or 256
 *   fwd_warps: warps per tile in the forward: 4 (8x8 pixel boxes, two pixels per
 *              lane) or 8 (8x4 boxes, one pixel per lane; fwd_batch 128 or 256)
 *   bwd_batch: instances staged per round in the backward: 32, 64 or 128
 *   bin_launch: batched solves only (cfgs_batch_iteration): 0 runs the binning (depth
 *              sort, emission, tile sort, tile ranges) as one launch per stage, 1 as one
 *              persistent cooperative launch with a bounded grid-wide wait between
 *              stages (same outputs)
 * All-zero fields mean the default {128, 4, 64, 0}; an unsupported combination makes the
 * call return CFGS_ERR_INVALID_ARGUMENT. */
typedef struct CfgsRenderSchedule {
  int32_t fwd_batch, fwd_warps, bwd_batch, bin_launch;
} CfgsRenderSchedule;

/* CFGS_OK when `schedule` is supported (zeros: the default), else
 * CFGS_ERR_INVALID_ARGUMENT; `resolved` (may be NULL) receives the schedule a call uses. */
int cfgs_render_schedule_check(const CfgsRenderSchedule* schedule, CfgsRenderSchedule* resolved);

/* GaussianRasterizationSettings (NamedTuple, 12 fields, order of
 * scene/gaussian_model_cf.py:811-824) plus the render schedule of the call. Tensor
 * fields are device pointers. */
typedef struct CfgsSettings {
  int32_t image_height;
  int32_t image_width;
  float tanfovx;
  float tanfovy;
  const float* bg;          /* [3]  background colour                               */
  float scale_modifier;
  const float* viewmatrix;  /* [16] world_view_transform                            */
  const float* projmatrix;  /* [16] full_proj_transform                             */
  int32_t sh_degree;        /* active SH degree, 0..3                               */
  const float* campos;      /* [3]  camera centre                                   */
  int32_t prefiltered;
  int32_t debug;            /* 1: synchronise and check after every kernel         */
  CfgsRenderSchedule schedule; /* launch shape of this call's render kernels (zeros: default) */
} CfgsSettings;

/* The per-Gaussian inputs of GaussianRasterizer.forward. Exactly one of
 * {shs, colors_precomp} and exactly one of {(scales, rotations), cov3D_precomp}
 * must be non-null (the Python layer raises before calling otherwise). */
typedef struct CfgsGaussians {
  int32_t num_gaussians;       /* N                                                */
  const float* means3D;        /* [N,3]                                            */
  const float* opacities;      /* [N]   (already sigmoid-activated)                */
  const float* shs;            /* [N,M,3] coefficient-major, channel last, or NULL */
  int32_t sh_coeffs;           /* M = shs.shape[1] (>= (sh_degree+1)^2)            */
  const float* colors_precomp; /* [N,3] or NULL                                    */
  const float* scales;         /* [N,3] or NULL (already exp-activated)            */
  const float* rotations;      /* [N,4] quaternion (r,x,y,z), or NULL              */
  const float* cov3D_precomp;  /* [N,6] (xx,xy,xz,yy,yz,zz), or NULL               */
} CfgsGaussians;

/* Gradient outputs of the backward pass (the 8 tensors upstream returns, in its
 * order). Every non-null array is fully overwritten (zeros for culled Gaussians). */
typedef struct CfgsGradients {
  float* dL_dmeans2D;   /* [N,3] d/d(NDC x, NDC y), third column 0             */
  float* dL_dcolors;    /* [N,3] d/d(per-Gaussian RGB)                        */
  float* dL_dopacity;   /* [N]                                                */
  float* dL_dmeans3D;   /* [N,3]                                              */
  float* dL_dcov3D;     /* [N,6]                                              */
  float* dL_dsh;        /* [N,M,3] or NULL when colors were precomputed        */
  float* dL_dscales;    /* [N,3] or NULL when cov3D was precomputed            */
  float* dL_drotations; /* [N,4] or NULL when cov3D was precomputed            */
} CfgsGradients;

/* Values the forward leaves in the image workspace; read with cfgs_read_counts(). */
typedef struct CfgsCounts {
  uint32_t num_rendered; /* K = total (Gaussian, tile) instances                 */
  uint32_t flags;        /* CFGS_FLAG_* bits                                     */
} CfgsCounts;

/* ---- workspace sizing (host functions, no device work) ---------------------- */

/* Per-Gaussian workspace ("geomBuffer" upstream). */
size_t cfgs_geom_bytes(int32_t num_gaussians);
/* Per-image workspace ("imageBuffer" upstream): counts, tile ranges, T_final,
 * contributor counts. */
size_t cfgs_image_bytes(int32_t image_width, int32_t image_height);
/* Per-instance workspace ("binningBuffer" upstream) for up to `capacity` instances. */
size_t cfgs_binning_bytes(int64_t capacity);
/* Scratch used by cfgs_backward for up to `capacity` instances: one 48-byte gradient
 * record per instance and one byte per instance that marks the records written (the
 * render backward writes only instances that reach a pixel; the others are zeros). */
size_t cfgs_backward_scratch_bytes(int64_t capacity);

/* Byte offsets of the arrays inside the workspaces, for inspection (tests, debugging;
 * upstream exposes the same buffers as opaque uint8 tensors).
 * geom  (14): xy float2, conic_op float4 (a,b,c,opacity), rgbd float4 (r,g,b,depth),
 *             rect uint2 (x0|y0<<16, x1|y1<<16), touched u32, offset u32 (first instance
 *             index), clamped u8, block_sums u32, depth_key u32[2][N], depth_val u32[2][N]
 *             (depth_val[1] = Gaussian ids in (depth, id) order), rank_sums u32,
 *             depth_counts u32, depth_totals u32, total bytes
 * image (6):  counts CfgsCounts, tile_count u32, tile_range u32[T+1], final_T f32,
 *             n_contrib u32, total bytes
 * binning (8): key u32[2][cap] (tile), gid u32[2][cap], pidx u32[2][cap],
 *             sorted_gid u32, sorted_pidx u32 (instance index), chunk_counts u32,
 *             totals u32, total bytes */
void cfgs_geom_layout(int32_t num_gaussians, size_t offsets[14]);
void cfgs_image_layout(int32_t image_width, int32_t image_height, size_t offsets[6]);
void cfgs_binning_layout(int64_t capacity, size_t offsets[8]);

/* ---- rasteriser forward, phase 1 ---------------------------------------------
 * Replaces the first half of upstream rasterize_gaussians (markVisible/preprocess
 * /InclusiveSum): projects every Gaussian (EWA), evaluates SH colour, computes the
 * screen radius and tile rectangle, and sums the tiles touched.
 * Writes radii[N] (0 = culled) and K into the image workspace. */
int cfgs_preprocess_forward(const CfgsSettings* settings, const CfgsGaussians* gaussians,
                            void* geom, void* image, int32_t* radii, void* stream);

/* Copies the CfgsCounts of an image workspace to host memory and synchronises
 * `stream`. (Upstream reads num_rendered back the same way.) */
int cfgs_read_counts(const void* image, CfgsCounts* counts_host, void* stream);

/* ---- rasteriser forward, phase 2 ---------------------------------------------
 * Replaces duplicateWithKeys / SortPairs / identifyTileRanges / render: sorts the
 * Gaussians by (view depth, id), emits the K (tile, Gaussian) instances in that order,
 * sorts them stably by tile — the order a stable sort of upstream's 64-bit key
 * (tile << 32 | depth bits) gives — and alpha-composites every 16x16 tile front to back.
 * out_color [3,H,W], out_depth [1,H,W], out_alpha [1,H,W]. `capacity` is the number
 * of instances the binning workspace holds; the device K is used, and if it exceeds
 * `capacity` the kernels raise CFGS_FLAG_CAPACITY_OVERFLOW and write nothing past it. */
int cfgs_render_forward(const CfgsSettings* settings, const CfgsGaussians* gaussians,
                        void* geom, void* image, void* binning, int64_t capacity,
                        float* out_color, float* out_depth, float* out_alpha, void* stream);

/* The two halves of cfgs_render_forward, for callers that time or schedule them
 * separately: depth sort + instance emission + tile sort + tile ranges
 * (duplicateWithKeys / SortPairs / identifyTileRanges upstream), then compositing
 * (renderCUDA upstream). */
int cfgs_bin_forward(const CfgsSettings* settings, const CfgsGaussians* gaussians, void* geom, void* image,
                     void* binning, int64_t capacity, void* stream);
int cfgs_composite_forward(const CfgsSettings* settings, int32_t num_gaussians, const void* geom,
                           const void* image, const void* binning, int64_t capacity, float* out_color,
                           float* out_depth, float* out_alpha, void* stream);

/* cfgs_bin_forward in two steps, so that the part that does not depend on K can run
 * while the host reads K: cfgs_depth_order (after cfgs_preprocess_forward: the depth
 * sort of the Gaussians, in the geom workspace) and cfgs_bin_instances (after it, with
 * the binning workspace sized for K: instance emission, tile sort, tile ranges).
 * cfgs_depth_order + cfgs_bin_instances = cfgs_bin_forward. */
int cfgs_depth_order(int32_t num_gaussians, void* geom, void* stream);
int cfgs_bin_instances(const CfgsSettings* settings, const CfgsGaussians* gaussians, void* geom, void* image,
                       void* binning, int64_t capacity, void* stream);

/* ---- rasteriser backward ------------------------------------------------------
 * Replaces upstream rasterize_gaussians_backward (render backward, computeCov2D
 * backward, preprocess backward). dL_dcolor [3,H,W]; dL_ddepth and dL_dalpha
 * [1,H,W] may be NULL (treated as zero). Per-pixel gradients are reduced per
 * (Gaussian, tile) inside each tile, written once per instance to `scratch`, and
 * summed per Gaussian in a fixed order: the result is deterministic. */
int cfgs_backward(const CfgsSettings* settings, const CfgsGaussians* gaussians,
                  const int32_t* radii, const void* geom, const void* image,
                  const void* binning, int64_t capacity, void* scratch,
                  const float* dL_dcolor, const float* dL_ddepth, const float* dL_dalpha,
                  const CfgsGradients* grads, void* stream);

/* The two halves of cfgs_backward: the per-tile render backward (renderCUDA backward
 * upstream) writing into `scratch` one record per instance that reaches a pixel and
 * marking it written (the marks are cleared first), then the per-Gaussian preprocess
 * backward (computeCov2DCUDA + preprocessCUDA backward upstream) summing the marked
 * records. */
int cfgs_render_backward(const CfgsSettings* settings, int32_t num_gaussians, const void* geom,
                         const void* image, const void* binning, int64_t capacity, void* scratch,
                         const float* dL_dcolor, const float* dL_ddepth, const float* dL_dalpha, void* stream);
int cfgs_preprocess_backward(const CfgsSettings* settings, const CfgsGaussians* gaussians,
                             const int32_t* radii, const void* geom, const void* image, int64_t capacity,
                             const void* scratch, const CfgsGradients* grads, void* stream);

/* ---- allocation-free backward ----------------------------------------------------
 * No counterpart in the reference: an addition of this library.
 *
 * For callers that cannot allocate device memory at the point they call the backward:
 * plugin hosts that give a plugin only its input and output buffers, and services that
 * must not allocate once serving has started. Same computation and outputs as
 * cfgs_backward, but the per-instance scratch is a fixed array inside the library, so
 * the caller passes no scratch buffer and nothing is allocated.
 *  - Limit: `capacity` (the binning capacity, >= K) at most
 *    CFGS_NOALLOC_MAX_INSTANCES instances; larger returns CFGS_ERR_TOO_LARGE.
 *  - Every GPU that loads the library holds the array (30.6 MiB) until the process exits.
 *  - The first call in a CUDA context looks up the array's device address (with the
 *    caller's device current) and caches it for that context; a context not seen before
 *    (a new one after cudaDeviceReset, or another context on the device) is looked up
 *    again. Make the first call of each context before any stream capture.
 *  - All calls share the one array and it keeps the last call's contents; each call
 *    clears what must start at zero (the per-instance "written" bytes) and writes every
 *    record it reads. Calls that overlap on the GPU race with each other: serialise
 *    them, e.g. on one stream. */
#define CFGS_NOALLOC_MAX_INSTANCES 655360
int cfgs_backward_noalloc(const CfgsSettings* settings, const CfgsGaussians* gaussians,
                          const int32_t* radii, const void* geom, const void* image,
                          const void* binning, int64_t capacity, const float* dL_dcolor,
                          const float* dL_ddepth, const float* dL_dalpha,
                          const CfgsGradients* grads, void* stream);

/* ---- diagnostics -----------------------------------------------------------------
 * No counterpart in the reference: a check of this library's failure handling.
 * The kernels that stage data by bulk or tensor copies wait for them on an mbarrier
 * with a bounded number of polls; a wait that gives up raises CFGS_FLAG_COPY_TIMEOUT and
 * the kernel returns, leaving the context usable. cfgs_diag_copy_timeout runs that same
 * wait, with `max_polls` polls (1 .. 2^22), on an mbarrier that no copy ever completes:
 * it writes the flags to `flags` (device uint32), synchronises `stream` and returns
 * CFGS_ERR_DEVICE_FLAG — the expected outcome — or CFGS_OK if the wait had completed. */
int cfgs_diag_copy_timeout(uint32_t max_polls, uint32_t* flags, void* stream);

/* ---- markVisible ---------------------------------------------------------------
 * Replaces upstream mark_visible (GaussianRasterizer.markVisible): visible[i] = 1
 * when the point's view-space z > 0.2. */
int cfgs_mark_visible(int32_t num_points, const float* means3D, const float* viewmatrix,
                      const float* projmatrix, uint8_t* visible, void* stream);

/* ---- CF-3DGS pose path --------------------------------------------------------
 * The pose is a tangent vector xi = (rho[3], phi[3]) retracted as exp(xi) * I, the
 * parametrisation of lietorch's LieGroupParameter(SE3) used by CFGaussianModel.init_RT
 * (scene/gaussian_model_cf.py:328-340); positions move as exp(xi).act(xyz)
 * (scene/gaussian_model_cf.py:123-133).
 *
 * cfgs_pose_apply: means_out[i] = R(xi) xyz[i] + t(xi); when cov_in/cov_out are
 * non-null also cov_out[i] = R cov_in[i] R^T (the rotate_cov form). */
int cfgs_pose_apply(int32_t num_points, const float* xi, const float* xyz,
                    const float* cov_in, float* means_out, float* cov_out, void* stream);

/* cfgs_pose_grad: dL/dxi [6] from dL/dmeans [N,3] (and, when both are non-null,
 * dL/dcov [N,6] of the rotated covariances cov_rot [N,6]) without materialising
 * per-Gaussian Jacobians: one pass forms the 6 (or 6+3) sums, the last block
 * folds them in a fixed order and applies the SE(3) left-Jacobian transpose.
 * `scratch` must hold cfgs_pose_scratch_bytes(N) bytes; `grad_out` is [6]. */
size_t cfgs_pose_scratch_bytes(int32_t num_points);
int cfgs_pose_grad(int32_t num_points, const float* xi, const float* xyz,
                   const float* dL_dmeans, const float* cov_rot, const float* dL_dcov,
                   void* scratch, float* grad_out, void* stream);

/* cfgs_pose_adam: one torch.optim.Adam step (no weight decay, no amsgrad) on `count`
 * independent 6-vectors xi[count][6], in place, with the step counts on the device:
 * state[count][16] = m(6), v(6), step(1), 3 unused. The operation sequence is that of
 * torch's default multi-tensor Adam for float32 CUDA tensors, with the float64
 * hyper-parameters rounded per use as torch does, so the steps match torch's. Mirrors
 * the optimiser the reference builds in training_setup_fix_position
 * (scene/gaussian_model_cf.py:303-326). */
int cfgs_pose_adam(int32_t count, float* xi, const float* grad, float* state, double lr,
                   double beta1, double beta2, double eps, void* stream);

/* ---- SSIM loss (pose-solve photometric loss) ---------------------------------------
 * Mean structural similarity of img1 against img2 ([C,H,W] float32, device), 11x11
 * Gaussian window (sigma 1.5), zero padding, one window per channel, C1 = 0.01^2,
 * C2 = 0.03^2: the ssim() of utils/loss_utils.py:33-58 and the _ssim of
 * trainer/losses.py:147-196 (size_average, no mask), which CF-3DGS weights as
 * (1 - lambda) L1 + lambda (1 - SSIM) (trainer/losses.py:98-136).
 * cfgs_ssim_forward writes the mean to ssim_mean (device float) and keeps in `scratch`
 * (cfgs_ssim_scratch_bytes) what the backward needs; cfgs_ssim_backward writes
 * dL/dimg1 = dL_dmean[0] * d mean / d img1 (img2 gets no gradient). Deterministic. */
size_t cfgs_ssim_scratch_bytes(int32_t channels, int32_t height, int32_t width);
int cfgs_ssim_forward(int32_t channels, int32_t height, int32_t width, const float* img1, const float* img2,
                      void* scratch, float* ssim_mean, void* stream);
int cfgs_ssim_backward(int32_t channels, int32_t height, int32_t width, const float* img1, const float* img2,
                       const void* scratch, const float* dL_dmean, float* dL_dimg1, void* stream);

/* ---- L1 photometric loss ------------------------------------------------------------
 * mean |x - target| over n floats (utils/loss_utils.py:15-16, trainer/losses.py:139-140),
 * of clamp(x, 0, 1) when clamp != 0 (the pose solve clamps the render before its loss:
 * scene/gaussian_model_cf.py:885). cfgs_l1_loss_forward writes the mean to loss (device
 * float; NaN for n = 0, as torch's mean) using `scratch` (cfgs_l1_loss_scratch_bytes) for
 * block partial sums (deterministic: fixed partition, float64 fold); when dL_dx is not
 * NULL it also writes, in the same pass, the gradient of the mean for an upstream
 * gradient of 1. cfgs_l1_loss_backward writes dL/dx = dL_dloss[0] * d mean / dx as
 * autograd forms it: (g / n) sign(c - target), zero where the clamp cuts (x < 0, x > 1). */
size_t cfgs_l1_loss_scratch_bytes(int64_t n);
int cfgs_l1_loss_forward(int64_t n, const float* x, const float* target, int32_t clamp, void* scratch, float* loss,
                         float* dL_dx, void* stream);
int cfgs_l1_loss_backward(int64_t n, const float* x, const float* target, int32_t clamp, const float* dL_dloss,
                          float* dL_dx, void* stream);

/* ---- frame initialisation (local Gaussians before each pose solve) ---------------------
 * kornia depth_to_3d (normalize_points=False; trainer/trainer.py:491): [H,W] depth ->
 * [H*W,3] camera-space points ((u - cx)/fx * d, (v - cy)/fy * d, d), row-major pixels. */
int cfgs_depth_to_points(int32_t height, int32_t width, const float* depth, float fx, float fy, float cx, float cy,
                         float* xyz, void* stream);
/* Device workspace of the two point-cloud operations below for num_points points. */
size_t cfgs_pointcloud_workspace_bytes(int64_t num_points);
/* simple-knn distCUDA2 (scene/gaussian_model_cf.py:194): dist2[i] = mean of the squared
 * distances from point i to its three nearest other points (FLT_MAX for missing ones).
 * Exact (Morton-ordered boxes with bounded pruning). */
int cfgs_knn3_mean_dist2(int64_t num_points, const float* xyz, void* workspace, float* dist2, void* stream);
/* Open3D voxel_down_sample (trainer/trainer.py:507): points (and colours, may be NULL)
 * of each occupied voxel floor((p - (min - s/2)) / s) averaged in float64 in input
 * order; out_xyz/out_rgb need room for num_points rows; *num_voxels receives the count
 * (voxels in increasing linear voxel index order). Synchronises `stream`. */
int cfgs_voxel_down_sample(int64_t num_points, const float* xyz, const float* rgb, double voxel_size,
                           void* workspace, float* out_xyz, float* out_rgb, int64_t* num_voxels, void* stream);

/* ---- Gaussian-parameter optimisation (global refinement, local fitting) ------------------
 * torch.optim.Adam over the parameter groups of GaussianModel.training_setup
 * (scene/gaussian_model_cf.py:242-266; eps 1e-15) in one launch: group k has numel[k]
 * float32 elements at params[k] with gradients grads[k] and moments exp_avg[k],
 * exp_avg_sq[k], learning rate lr[k]; `step` is the step count after this step. The
 * operation sequence is torch's multi-tensor Adam, so results are bit-identical. */
int cfgs_gaussian_adam(int32_t num_groups, float* const* params, const float* const* grads, float* const* exp_avg,
                       float* const* exp_avg_sq, const int64_t* numel, const double* lr, double beta1, double beta2,
                       double eps, int64_t step, void* stream);
/* add_densification_stats (scene/gaussian_model_cf.py:716-719) with the visibility filter
 * radii > 0: grad_accum += |dL/dmeans2D[:, :2]|, denom += 1. */
int cfgs_densify_stats(int64_t num_gaussians, const int32_t* radii, const float* grad_means2D, float* grad_accum,
                       float* denom, void* stream);
/* densify_and_prune (scene/gaussian_model_cf.py:628-694), in two steps. cfgs_densify_plan
 * classifies every Gaussian and returns counts = {kept originals, kept clones, split
 * points, kept children per copy} (synchronises `stream`); cfgs_densify_write then writes
 * one array of the new model, rows = counts[0] + counts[1] + 2 counts[3] in the
 * reference's order (kept originals, kept clones, children copy 0, children copy 1):
 * role 0 copies a parameter array of `width` floats per row, 1 an Adam moment (zero for
 * new rows), 2 the positions and 3 the scalings (split children computed from xyz,
 * scaling, rotation and the standard-normal draws z [2][counts[2]][3]). */
size_t cfgs_densify_workspace_bytes(int64_t num_gaussians);
int cfgs_densify_plan(int64_t num_gaussians, const float* grad_accum, const float* denom, const float* scaling,
                      const float* opacity, float max_grad, float min_opacity, float extent, float percent_dense,
                      int32_t prune_big, void* workspace, int64_t counts[4], void* stream);
int cfgs_densify_write(int64_t num_gaussians, void* workspace, const int64_t counts[4], int32_t width,
                       const float* in, float* out, int32_t role, const float* xyz, const float* scaling,
                       const float* rotation, const float* z, void* stream);

/* ---- batched pose solves ----------------------------------------------------------
 * Many CF-3DGS pose solves (trainer/cf3dgs_trainer.py:261-285), each with its own
 * Gaussians, camera and resolution, advance together: one call runs one Adam iteration
 * of every solve with one launch per stage (preprocess, scan, depth sort, emission,
 * tile sort, tile ranges, composite, render backward with the RGB L1 image gradient formed in-kernel, pose-only
 * preprocess backward, per-solve pose update). Nothing synchronises, so a sequence of
 * iterations can be captured in a CUDA graph. Per solve the arithmetic is that of the
 * single-solve path (cfgs_pose_apply -> rasteriser -> cfgs_pose_grad -> cfgs_pose_adam).
 *
 * Layout: solve s owns Gaussian slots [gauss_base, gauss_base + N_s) with gauss_base a
 * multiple of 256 (slots up to the next multiple are padding), tiles
 * [tile_base, tile_base + T_s) and pixels [pix_base, pix_base + W_s H_s); per-pixel
 * images of s start at pix_base (colour and target at 3 * pix_base, [3, H_s, W_s]). */
typedef struct CfgsBatchScene {   /* host description of one solve */
  int32_t image_width, image_height;
  float tanfovx, tanfovy;
  const float* viewmatrix;  /* device [16] */
  const float* projmatrix;  /* device [16] */
  const float* campos;      /* device [3]  */
  const float* bg;          /* device [3]  */
  int32_t sh_degree, sh_coeffs;
  int32_t num_gaussians;
} CfgsBatchScene;

typedef struct CfgsBatchPlan {    /* sizes of a batch, filled by cfgs_batch_plan */
  int32_t num_scenes;
  int32_t num_blocks;        /* 256-wide Gaussian blocks = gauss_slots / 256     */
  int64_t gauss_slots;
  int32_t num_tiles;
  int32_t pad_;
  int64_t num_pixels;
  size_t desc_bytes;         /* scene table (device copy of the host table)      */
  size_t pose_state_bytes;   /* per-solve pose state                             */
  size_t geom_bytes, image_bytes;
} CfgsBatchPlan;

/* Host-only: computes the plan and, when the output pointers are non-null, the host
 * images of the scene table (desc_host, plan.desc_bytes), the block->solve map
 * (block_scene_host, num_blocks int32) and the tile->solve map (tile_scene_host,
 * num_tiles int32), plus per-solve bases (gauss_base, tile_base: int32 [S];
 * pix_base: int64 [S]). `pose_states_device` is where the caller will keep the pose
 * states (plan.pose_state_bytes) on the device. */
int cfgs_batch_plan(int32_t num_scenes, const CfgsBatchScene* scenes, const void* pose_states_device,
                    CfgsBatchPlan* plan, void* desc_host, int32_t* block_scene_host, int32_t* tile_scene_host,
                    int32_t* gauss_base, int32_t* tile_base, int64_t* pix_base);

typedef struct CfgsBatchArgs {    /* device pointers of one batch */
  int32_t num_scenes, num_blocks, num_tiles, pad_;
  int64_t gauss_slots, capacity;
  const void* descs;              /* scene table, plan.desc_bytes               */
  const int32_t* block_scene;
  const int32_t* tile_scene;
  const float* means3D;           /* [slots,3] un-posed positions              */
  const float* opacities;         /* [slots]                                   */
  const float* shs;               /* [slots,M,3] (M = the solves' sh_coeffs)   */
  const float* scales;            /* [slots,3]                                 */
  const float* rotations;         /* [slots,4]                                 */
  const float* target;            /* [3 * num_pixels]                          */
  float* color;                   /* [3 * num_pixels] render of the iteration  */
  int32_t* radii;                 /* [slots]                                   */
  void* geom;                     /* plan.geom_bytes                           */
  void* image;                    /* plan.image_bytes                          */
  void* binning;                  /* cfgs_binning_bytes(capacity)              */
  void* scratch;                  /* cfgs_backward_scratch_bytes(capacity)     */
  double* pose_partials;          /* [num_blocks][9]                           */
  float* xi;                      /* [S][6] tangents, updated in place         */
  float* adam_state;              /* [S][16] (cfgs_pose_adam layout)           */
  void* pose_states;              /* plan.pose_state_bytes                     */
  double lr, beta1, beta2, eps;
  CfgsRenderSchedule schedule;    /* render kernels' launch shape (zeros: default) */
  int32_t sh_degree_bound;        /* 1 + the largest SH degree of the solves; 0: not stated.
                                     1 (every solve SH degree 0, colour independent of the
                                     view, so only the 2D-mean and conic gradient sums reach
                                     the pose) lets the render backward form those sums
                                     alone; any other value forms all of them */
  int32_t pad2_;
} CfgsBatchArgs;

/* Sets every solve's pose state from xi (call once before the first iteration). */
int cfgs_batch_init(const CfgsBatchArgs* args, void* stream);
/* One Adam iteration of every solve. K (all solves' tile instances together) above
 * `capacity` raises CFGS_FLAG_CAPACITY_OVERFLOW in the image workspace's counts (read
 * with cfgs_read_counts); that iteration's update is then skipped. */
int cfgs_batch_iteration(const CfgsBatchArgs* args, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CFGS_H */
