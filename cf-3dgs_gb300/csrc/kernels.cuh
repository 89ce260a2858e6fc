// Kernel argument blocks and launchers shared by the drop-in entry points and the
// batched pose-solve engine. Each launcher is defined in the translation unit that
// holds its kernel (the forward ones are compiled without FMA contraction).
#pragma once

#include "cfgs_internal.cuh"

namespace cfgs {

template <class Scenes>
struct PreArgs {
  Scenes scenes;
  CfgsGaussians g;  // pointers index the global (padded) Gaussian arrays
  GeomView geom;
  CfgsCounts* counts;
  int32_t* radii;
  int64_t total_slots;  // Gaussian slots covered by the launch (padded in batches)
};

// Binning: depth sort, emission in depth order, tile sort, tile ranges.
template <class Scenes>
struct BinArgs {
  Scenes scenes;
  int64_t total_slots;
  GeomView geom;
  BinningView bin;
  int64_t cap;
  CfgsCounts* counts;
  int64_t num_tiles;  // all scenes' tiles
  uint32_t* tile_count;
  uint32_t* tile_range;
};

template <class Scenes>
struct EmitArgs {
  Scenes scenes;
  int64_t total_slots;
  const uint32_t* order;      // Gaussians in (depth, id) order
  const uint32_t* rank_sums;  // instances per 256 of them (exclusive prefix when rank_scanned)
  bool rank_scanned;          // k_rank_scan ran (rank_scan_needed)
  GeomView geom;
  BinningView bin;
  int64_t cap;
  CfgsCounts* counts;
};

template <class Scenes>
struct RenderArgs {
  Scenes scenes;
  const uint32_t* tile_range;
  const uint32_t* sorted_gid;
  const float2* xy;
  const float4* conic_op;
  const float4* rgbd;
  float* final_T;
  uint32_t* n_contrib;
  float* out_color;
  float* out_depth;
  float* out_alpha;
  int64_t cap;
  const CfgsCounts* counts;
  CfgsRenderSchedule sched;  // resolved launch shape (resolve_schedule)
};

// Render backward. The per-pixel image gradient comes either from dL_dcolor (layout
// of out_color) or, when `target` is set, from the RGB L1 loss of the clamped render,
// mean |clamp(color, 0, 1) - target| over the scene's 3*W*H values, formed in-kernel
// exactly as autograd forms it: sign(clamp(c) - t) * [0 <= c <= 1] * (1 / numel).
template <class Scenes>
struct RenderBwdArgs {
  Scenes scenes;
  const uint32_t* tile_range;
  const uint32_t* sorted_gid;
  const uint32_t* sorted_pidx;
  const float2* xy;
  const float4* conic_op;
  const float4* rgbd;
  const float* final_T;
  const uint32_t* n_contrib;
  const float* dL_dcolor;
  const float* dL_ddepth;
  const float* dL_dalpha;
  const float* color;   // forward output (fused L1 only)
  const float* target;  // fused L1 target, or NULL
  float4* records;
  uint8_t* written;     // per instance: 1 when its record was written (zeroed beforehand)
  int64_t cap;
  const CfgsCounts* counts;
  CfgsRenderSchedule sched;  // resolved launch shape (resolve_schedule)
  bool geom_only;            // form only the 2D-mean and conic sums (batched SH-degree-0 pose solves)
};

template <class Scenes>
struct PreBwdArgs {
  Scenes scenes;
  CfgsGaussians g;
  const int32_t* radii;
  GeomView geom;
  const float4* records;
  const uint8_t* written;  // records whose byte is 0 are exact zeros and are not read
  CfgsGradients out;
  int64_t total_slots;
  int64_t cap;
  const CfgsCounts* counts;
  double* pose_partials;  // pose-only form: [block][9] float64 sums; NULL for the full backward
  bool sh_bulk;           // degree-3 SH of each block moved by bulk copies (16-byte aligned arrays)
  uint32_t* flags;        // CFGS_FLAG_COPY_TIMEOUT
};

template <class Scenes>
void launch_preprocess(const PreArgs<Scenes>& a, int blocks, cudaStream_t st);
void launch_scan(uint32_t* block_sums, int num_blocks, CfgsCounts* counts, cudaStream_t st);
template <class Scenes>
int launch_binning(const BinArgs<Scenes>& a, cudaStream_t st);
template <class Scenes>
int launch_binning_persistent(const BinArgs<Scenes>& a, GridBarrier* barrier, cudaStream_t st);
int sort_pairs(uint32_t* keys[2], uint32_t* vals[2], int64_t n, int bits, uint32_t* chunk_counts, uint32_t* totals,
               cudaStream_t st, int* result);
template <class Scenes>
void launch_render_fwd(const RenderArgs<Scenes>& a, int tiles, cudaStream_t st);
template <class Scenes>
void launch_render_bwd(const RenderBwdArgs<Scenes>& a, int tiles, cudaStream_t st);
template <class Scenes>
void launch_preprocess_bwd(const PreBwdArgs<Scenes>& a, int blocks, cudaStream_t st);
// The schedule a call uses: zeros become the default {128, 4, 64}; false when the
// combination is not one the render kernels are instantiated for.
bool resolve_schedule(const CfgsRenderSchedule& in, CfgsRenderSchedule* out);

void launch_batch_pose_init(int count, const float* xi, const float* adam_state, PoseState* states, double b1,
                            double b2, cudaStream_t st);
void launch_batch_pose_update(int count, const SceneDesc* descs, const double* partials, float* xi,
                              float* adam_state, PoseState* states, const CfgsCounts* counts, int64_t cap, double lr,
                              double b1, double b2, double eps, cudaStream_t st);

}  // namespace cfgs
