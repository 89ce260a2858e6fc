// Batched CF-3DGS pose solves: planning of the packed layout and one Adam iteration of
// every solve, one launch per stage. The kernels are the drop-in path's kernels
// instantiated for a scene table, so every solve computes exactly what it computes
// alone.
#include "cfgs_internal.cuh"
#include "kernels.cuh"

using namespace cfgs;

extern "C" int cfgs_batch_plan(int32_t num_scenes, const CfgsBatchScene* scenes, const void* pose_states_device,
                               CfgsBatchPlan* plan, void* desc_host, int32_t* block_scene_host,
                               int32_t* tile_scene_host, int32_t* gauss_base, int32_t* tile_base, int64_t* pix_base) {
  if (num_scenes <= 0 || !scenes || !plan) return CFGS_ERR_INVALID_ARGUMENT;
  int64_t slots = 0, pixels = 0;
  int64_t tiles = 0;
  for (int s = 0; s < num_scenes; ++s) {
    const CfgsBatchScene& c = scenes[s];
    if (c.image_width <= 0 || c.image_height <= 0 || c.num_gaussians < 0 || c.sh_degree < 0 || c.sh_degree > 3 ||
        c.sh_coeffs < (c.sh_degree + 1) * (c.sh_degree + 1) || c.image_width > 65535 * kTileX ||
        c.image_height > 65535 * kTileY)
      return CFGS_ERR_INVALID_ARGUMENT;
    const int gx = (c.image_width + kTileX - 1) / kTileX, gy = (c.image_height + kTileY - 1) / kTileY;
    if (gauss_base) gauss_base[s] = (int32_t)slots;
    if (tile_base) tile_base[s] = (int32_t)tiles;
    if (pix_base) pix_base[s] = pixels;
    if (desc_host) {
      SceneDesc& d = static_cast<SceneDesc*>(desc_host)[s];
      d = SceneDesc{};
      d.W = c.image_width;
      d.H = c.image_height;
      d.grid_x = gx;
      d.grid_y = gy;
      d.tile_base = (int32_t)tiles;
      d.num_tiles = gx * gy;
      d.gauss_base = (int32_t)slots;
      d.num_gaussians = c.num_gaussians;
      d.pix_base = pixels;
      d.sh_degree = c.sh_degree;
      d.sh_coeffs = c.sh_coeffs;
      d.prefiltered = 0;
      d.tanfovx = c.tanfovx;
      d.tanfovy = c.tanfovy;
      d.focal_x = (float)c.image_width / (2.0f * c.tanfovx);
      d.focal_y = (float)c.image_height / (2.0f * c.tanfovy);
      d.scale_modifier = 1.0f;
      d.inv_numel = 1.0f / (float)(3.0 * (double)c.image_width * (double)c.image_height);
      d.V = c.viewmatrix;
      d.P = c.projmatrix;
      d.campos = c.campos;
      d.bg = c.bg;
      d.pose = pose_states_device ? static_cast<const PoseState*>(pose_states_device) + s : nullptr;
    }
    const int64_t nblk = ((int64_t)c.num_gaussians + kPreprocessBlock - 1) / kPreprocessBlock;
    if (block_scene_host)
      for (int64_t b = 0; b < nblk; ++b) block_scene_host[slots / kPreprocessBlock + b] = s;
    if (tile_scene_host)
      for (int64_t t = 0; t < (int64_t)gx * gy; ++t) tile_scene_host[tiles + t] = s;
    slots += nblk * kPreprocessBlock;
    tiles += (int64_t)gx * gy;
    pixels += (int64_t)c.image_width * c.image_height;
  }
  if (slots > 0x7fffff00ll || tiles > 0x7fffffffll) return CFGS_ERR_TOO_LARGE;
  plan->num_scenes = num_scenes;
  plan->gauss_slots = slots;
  plan->num_blocks = (int32_t)(slots / kPreprocessBlock);
  plan->num_tiles = (int32_t)tiles;
  plan->num_pixels = pixels;
  plan->desc_bytes = sizeof(SceneDesc) * (size_t)num_scenes;
  plan->pose_state_bytes = sizeof(PoseState) * (size_t)num_scenes;
  plan->geom_bytes = GeomLayout((int32_t)slots).total;
  // The image workspace of a batch has the layout of one (16 T) x 16 strip image: T tile
  // entries and 256 T >= num_pixels per-pixel entries.
  plan->image_bytes = ImageLayout(kTileX * (int32_t)tiles, kTileY).total;
  return CFGS_OK;
}

namespace {

struct BatchViews {
  ImageView iv;
  GeomView gv;
  BinningView bv;
  SceneTable table;
};

// The batch image workspace reuses the single-image layout of a (16*T) x 16 strip,
// whose tile arrays have T entries; final_T and n_contrib are sized for the batch's
// pixels (cfgs_batch_plan reserves them).
BatchViews views(const CfgsBatchArgs* a) {
  BatchViews v;
  const int32_t w = kTileX * a->num_tiles;
  ImageLayout IL(w, kTileY);
  char* b = static_cast<char*>(a->image);
  v.iv.counts = reinterpret_cast<CfgsCounts*>(b + IL.header);
  v.iv.tile_count = reinterpret_cast<uint32_t*>(b + IL.tile_count);
  v.iv.tile_range = reinterpret_cast<uint32_t*>(b + IL.tile_range);
  v.iv.final_T = reinterpret_cast<float*>(b + IL.final_T);
  // n_contrib follows final_T's batch-sized array
  v.iv.n_contrib = reinterpret_cast<uint32_t*>(b + IL.n_contrib);
  v.gv = GeomView(a->geom, (int32_t)a->gauss_slots);
  v.bv = BinningView(a->binning, a->capacity);
  v.table.d = static_cast<const SceneDesc*>(a->descs);
  v.table.block_scene = a->block_scene;
  v.table.tile_scene = a->tile_scene;
  return v;
}

bool args_ok(const CfgsBatchArgs* a) {
  return a && a->num_scenes > 0 && a->num_blocks > 0 && a->num_tiles > 0 && a->descs && a->block_scene &&
         a->tile_scene && a->means3D && a->opacities && a->shs && a->scales && a->rotations && a->target &&
         a->color && a->radii && a->geom && a->image && a->binning && a->scratch && a->pose_partials && a->xi &&
         a->adam_state && a->pose_states && a->capacity >= 0 && a->capacity <= 0x7fffffffll &&
         a->gauss_slots == (int64_t)a->num_blocks * kPreprocessBlock;
}

}  // namespace

extern "C" int cfgs_batch_init(const CfgsBatchArgs* a, void* stream) {
  if (!args_ok(a)) return CFGS_ERR_INVALID_ARGUMENT;
  launch_batch_pose_init(a->num_scenes, a->xi, a->adam_state, static_cast<PoseState*>(a->pose_states), a->beta1,
                         a->beta2, (cudaStream_t)stream);
  CFGS_CHECK_LAUNCH(0, stream);
  return CFGS_OK;
}

extern "C" int cfgs_batch_iteration(const CfgsBatchArgs* a, void* stream) {
  if (!args_ok(a)) return CFGS_ERR_INVALID_ARGUMENT;
  CfgsRenderSchedule sched;
  if (!resolve_schedule(a->schedule, &sched)) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  BatchViews v = views(a);
  // the counts and the one-launch binning's barrier state (the header's first 256 bytes)
  if (cudaMemsetAsync(v.iv.counts, 0, 256, st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  if (cudaMemsetAsync(v.iv.tile_count, 0, sizeof(uint32_t) * (size_t)a->num_tiles, st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;

  CfgsGaussians g{};
  g.num_gaussians = (int32_t)a->gauss_slots;
  g.means3D = a->means3D;
  g.opacities = a->opacities;
  g.shs = a->shs;
  g.scales = a->scales;
  g.rotations = a->rotations;

  PreArgs<SceneTable> pa;
  pa.scenes = v.table;
  pa.g = g;
  pa.geom = v.gv;
  pa.counts = v.iv.counts;
  pa.radii = a->radii;
  pa.total_slots = a->gauss_slots;
  launch_preprocess(pa, a->num_blocks, st);
  launch_scan(v.gv.block_sums, a->num_blocks, v.iv.counts, st);

  BinArgs<SceneTable> ba;
  ba.scenes = v.table;
  ba.total_slots = a->gauss_slots;
  ba.geom = v.gv;
  ba.bin = v.bv;
  ba.cap = a->capacity;
  ba.counts = v.iv.counts;
  ba.num_tiles = a->num_tiles;
  ba.tile_count = v.iv.tile_count;
  ba.tile_range = v.iv.tile_range;
  GridBarrier* barrier = reinterpret_cast<GridBarrier*>(reinterpret_cast<char*>(v.iv.counts) + kGridBarrierOffset);
  int status = sched.bin_launch ? launch_binning_persistent(ba, barrier, st) : launch_binning(ba, st);
  if (status != CFGS_OK) return status;

  RenderArgs<SceneTable> ra;
  ra.scenes = v.table;
  ra.tile_range = v.iv.tile_range;
  ra.sorted_gid = v.bv.sorted_gid;
  ra.xy = v.gv.xy;
  ra.conic_op = v.gv.conic_op;
  ra.rgbd = v.gv.rgbd;
  ra.final_T = v.iv.final_T;
  ra.n_contrib = v.iv.n_contrib;
  ra.out_color = a->color;
  ra.out_depth = nullptr;
  ra.out_alpha = nullptr;
  ra.cap = a->capacity;
  ra.counts = v.iv.counts;
  ra.sched = sched;
  launch_render_fwd(ra, a->num_tiles, st);

  RenderBwdArgs<SceneTable> rb;
  rb.scenes = v.table;
  rb.tile_range = v.iv.tile_range;
  rb.sorted_gid = v.bv.sorted_gid;
  rb.sorted_pidx = v.bv.sorted_pidx;
  rb.xy = v.gv.xy;
  rb.conic_op = v.gv.conic_op;
  rb.rgbd = v.gv.rgbd;
  rb.final_T = v.iv.final_T;
  rb.n_contrib = v.iv.n_contrib;
  rb.dL_dcolor = nullptr;
  rb.dL_ddepth = nullptr;
  rb.dL_dalpha = nullptr;
  rb.color = a->color;
  rb.target = a->target;
  const ScratchLayout SL(a->capacity);
  rb.records = reinterpret_cast<float4*>(static_cast<char*>(a->scratch) + SL.records);
  rb.written = reinterpret_cast<uint8_t*>(static_cast<char*>(a->scratch) + SL.written);
  if (a->capacity > 0 && cudaMemsetAsync(rb.written, 0, (size_t)a->capacity, st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  rb.cap = a->capacity;
  rb.counts = v.iv.counts;
  rb.sched = sched;
  // Every solve SH degree 0: colour does not depend on the view, so the colour and
  // opacity sums never reach the pose and the render backward forms the 2D-mean and
  // conic sums alone (the same bits for those); the records' other terms are zeros.
  rb.geom_only = a->sh_degree_bound == 1;
  launch_render_bwd(rb, a->num_tiles, st);

  PreBwdArgs<SceneTable> pb;
  pb.scenes = v.table;
  pb.g = g;
  pb.radii = a->radii;
  pb.geom = v.gv;
  pb.records = rb.records;
  pb.written = rb.written;
  pb.out = CfgsGradients{};
  pb.total_slots = a->gauss_slots;
  pb.cap = a->capacity;
  pb.counts = v.iv.counts;
  pb.pose_partials = a->pose_partials;
  pb.flags = &v.iv.counts->flags;
  pb.sh_bulk = false;  // batched solves carry degree-0 colours
  launch_preprocess_bwd(pb, a->num_blocks, st);

  launch_batch_pose_update(a->num_scenes, v.table.d, a->pose_partials, a->xi, a->adam_state,
                           static_cast<PoseState*>(a->pose_states), v.iv.counts, a->capacity, a->lr, a->beta1,
                           a->beta2, a->eps, st);
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}
