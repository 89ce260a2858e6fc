// Forward phase 3: front-to-back alpha compositing of every 16x16 tile over its
// depth-sorted instance list.
//
// The kernel is a template over the scene accessor (one scene for the drop-in path, a
// descriptor table for batched solves); the arithmetic is the same for both.
// Compiled with -fmad=false; the fmaf() calls are the only fused operations, and the
// CPU oracle performs the same sequence.
#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

// Launch schedules (cfgs_set_render_schedule): kRenderBatch instances staged per round
// and 4 or 8 warps per tile. Every schedule gives bit-identical outputs: each pixel sees
// the same instances in the same order with the same arithmetic.
constexpr int kRenderBatch = 128;

// Front-to-back state of a lane's two pixels (.x: row r, .y: row r + 4) and one
// compositing step of both: the published loop body per pixel, with the exponential
// skipped below the alpha threshold (exact, see alpha_threshold). The arithmetic runs on
// packed pairs (bit-identical to the scalar operations); each pixel's decisions are its
// own, and a pixel that does not take the step keeps its state.
struct PairFwd {
  float2 T, C0, C1, C2, D;
  uint32_t last0, last1;
  bool done0, done1;
};

template <bool DEPTH>
__device__ __forceinline__ void composite_pair(PairFwd& p, float pxf, float2 pyf, const float4& xyt, const float4& co,
                                               const float4* s_rgbd, int j, uint32_t pos1) {
  const float2 power = gauss_power2(co.x, co.y, co.z, xyt.x - pxf, sub2(splat2(xyt.y), pyf));
  bool a0 = !p.done0 && !(power.x > 0.0f || power.x < xyt.z);
  bool a1 = !p.done1 && !(power.y > 0.0f || power.y < xyt.z);
  if (!(a0 || a1)) return;
  float2 alpha = mul2(splat2(co.w), exp_ref_inrange2(power));
  alpha.x = fminf(CFGS_ALPHA_MAX, alpha.x);
  alpha.y = fminf(CFGS_ALPHA_MAX, alpha.y);
  a0 = a0 && !(alpha.x < CFGS_ALPHA_MIN);
  a1 = a1 && !(alpha.y < CFGS_ALPHA_MIN);
  if (!(a0 || a1)) return;
  const float2 test_T = mul2(p.T, sub2(splat2(1.0f), alpha));
  const bool end0 = a0 && test_T.x < CFGS_T_MIN, end1 = a1 && test_T.y < CFGS_T_MIN;
  p.done0 = p.done0 || end0;
  p.done1 = p.done1 || end1;
  const bool u0 = a0 && !end0, u1 = a1 && !end1;
  if (!(u0 || u1)) return;
  const float4 c = s_rgbd[j];
  const float2 w = mul2(alpha, p.T);
  const float2 C0 = fma2(splat2(c.x), w, p.C0);
  const float2 C1 = fma2(splat2(c.y), w, p.C1);
  const float2 C2 = fma2(splat2(c.z), w, p.C2);
  const float2 D = DEPTH ? fma2(splat2(c.w), w, p.D) : p.D;
  if (u0) {
    p.C0.x = C0.x;
    p.C1.x = C1.x;
    p.C2.x = C2.x;
    p.D.x = D.x;
    p.T.x = test_T.x;
    p.last0 = pos1;
  }
  if (u1) {
    p.C0.y = C0.y;
    p.C1.y = C1.y;
    p.C2.y = C2.y;
    p.D.y = D.y;
    p.T.y = test_T.y;
    p.last1 = pos1;
  }
}

// One block of 32 WARPS threads per 16x16 tile. With 4 warps, warp w covers the 8x8
// pixel box (8 (w & 1), 8 (w >> 1)) and each lane two pixels of it, rows r and r + 4;
// with 8 warps, warp w covers the 8x4 box (8 (w & 1), 4 (w >> 1)) and each lane one
// pixel (the pair's second pixel is never inside). Batches of BATCH instances are
// gathered into shared memory (per-Gaussian data stays L2-resident).
// Two exact shortcuts skip work whose outcome is known: each warp keeps only the
// instances whose alpha >= 1/255 ellipse can reach its box (box_may_contribute, one test
// per instance and warp), and a pixel skips the exponential when the exponent lies
// below the instance's alpha_threshold. Neither changes a decision of the published
// algorithm, so every output — contributor counts included, which count positions in
// the tile's list — is what the plain per-pixel loop gives. Compositing runs front to
// back; a warp stops when its pixels are saturated and the block when all are.
template <class Scenes, int BATCH, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_render_fwd(RenderArgs<Scenes> a) {
  static_assert(BATCH % 32 == 0 && (WARPS == 4 || WARPS == 8), "whole ballot words; 8x8 or 8x4 warp boxes");
  constexpr int kThreads = 32 * WARPS;
  constexpr int kBoxRows = WARPS == 4 ? 8 : 4;
  __shared__ float4 s_xyt[BATCH];   // (x, y, alpha threshold, -)
  __shared__ float4 s_co[BATCH];    // (ca, cb, cc, opacity)
  __shared__ float4 s_rgbd[BATCH];
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const int tile = blockIdx.x;
  const SceneDesc& sd = a.scenes.for_tile(tile);
  const int lt = tile - sd.tile_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bx0 = (lt % sd.grid_x) * kTileX + (warp & 1) * 8;
  const int by0 = (lt / sd.grid_x) * kTileY + (warp >> 1) * kBoxRows;
  const int px = bx0 + (lane & 7), py0 = by0 + (lane >> 3), py1 = py0 + 4;
  const float bxf0 = (float)bx0, bxf1 = (float)(bx0 + 7), byf0 = (float)by0, byf1 = (float)(by0 + kBoxRows - 1);
  const bool in0 = px < sd.W && py0 < sd.H, in1 = WARPS == 4 && px < sd.W && py1 < sd.H;
  const float pxf = (float)px, pyf0 = (float)py0, pyf1 = (float)py1;
  const uint32_t lo = a.tile_range[tile];
  const int n = (int)(a.tile_range[tile + 1] - lo);
  PairFwd pp{splat2(1.0f), splat2(0.0f), splat2(0.0f), splat2(0.0f), splat2(0.0f), 0u, 0u, !in0, !in1};
  const float2 pyf = make_float2(pyf0, pyf1);
  for (int base = 0; base < n; base += BATCH) {
    if (__syncthreads_count(pp.done0 && pp.done1) == kThreads) break;
#pragma unroll
    for (int j = threadIdx.x; j < BATCH; j += kThreads) {
      const int i = base + j;
      if (i < n) {
        uint32_t g = a.sorted_gid[lo + i];
        float2 m = a.xy[g];
        float4 co = a.conic_op[g];
        s_xyt[j] = make_float4(m.x, m.y, alpha_threshold(co.w), 0.0f);
        s_co[j] = make_float4(-0.5f * co.x, -co.y, -0.5f * co.z, co.w);
        s_rgbd[j] = a.rgbd[g];
      }
    }
    __syncthreads();
    const int cnt = min(BATCH, n - base);
    uint32_t keep[BATCH / 32];
#pragma unroll
    for (int r = 0; r < BATCH / 32; ++r) {
      const int j = r * 32 + lane;
      bool k = false;
      if (j < cnt) {
        const float4 xyt = s_xyt[j];
        const float4 co = s_co[j];
        k = box_may_contribute(make_float2(xyt.x, xyt.y), co.x, co.y, co.z, xyt.z, bxf0, bxf1, byf0, byf1);
      }
      keep[r] = __ballot_sync(0xffffffffu, k);
    }
#pragma unroll
    for (int r = 0; r < BATCH / 32; ++r) {
      if (__all_sync(0xffffffffu, pp.done0 && pp.done1)) break;
      uint32_t mk = keep[r];
      while (mk) {
        const int j = r * 32 + __ffs(mk) - 1;
        mk &= mk - 1;
        const float4 xyt = s_xyt[j];
        const float4 co = s_co[j];
        const uint32_t pos1 = (uint32_t)(base + j + 1);
        composite_pair<!Scenes::kBatched>(pp, pxf, pyf, xyt, co, s_rgbd, j, pos1);  // batches ask for no depth
      }
    }
  }
  const size_t HW = (size_t)sd.W * sd.H;
  float* col = a.out_color + 3 * (size_t)sd.pix_base;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int py = q ? py1 : py0;
    if (!(q ? in1 : in0)) continue;
    const float T = q ? pp.T.y : pp.T.x;
    const size_t pix = (size_t)py * sd.W + px;
    const size_t gp = (size_t)sd.pix_base + pix;
    a.final_T[gp] = T;
    a.n_contrib[gp] = q ? pp.last1 : pp.last0;
    col[pix] = fmaf(T, __ldg(sd.bg + 0), q ? pp.C0.y : pp.C0.x);
    col[HW + pix] = fmaf(T, __ldg(sd.bg + 1), q ? pp.C1.y : pp.C1.x);
    col[2 * HW + pix] = fmaf(T, __ldg(sd.bg + 2), q ? pp.C2.y : pp.C2.x);
    if (a.out_depth) a.out_depth[gp] = q ? pp.D.y : pp.D.x;
    if (a.out_alpha) a.out_alpha[gp] = 1.0f - T;
  }
}

template <class Scenes>
void launch_render_fwd(const RenderArgs<Scenes>& a, int tiles, cudaStream_t st) {
  const CfgsRenderSchedule& rs = a.sched;
  if (rs.fwd_warps == 8) {
    if (rs.fwd_batch == 256) k_render_fwd<Scenes, 256, 8><<<tiles, 256, 0, st>>>(a);
    else k_render_fwd<Scenes, 128, 8><<<tiles, 256, 0, st>>>(a);
  } else {
    if (rs.fwd_batch == 64) k_render_fwd<Scenes, 64, 4><<<tiles, 128, 0, st>>>(a);
    else if (rs.fwd_batch == 256) k_render_fwd<Scenes, 256, 4><<<tiles, 128, 0, st>>>(a);
    else k_render_fwd<Scenes, kRenderBatch, 4><<<tiles, 128, 0, st>>>(a);
  }
}
template void launch_render_fwd<SingleScene>(const RenderArgs<SingleScene>&, int, cudaStream_t);
template void launch_render_fwd<SceneTable>(const RenderArgs<SceneTable>&, int, cudaStream_t);

bool resolve_schedule(const CfgsRenderSchedule& in, CfgsRenderSchedule* out) {
  if (in.bin_launch != 0 && in.bin_launch != 1) return false;
  if (in.fwd_batch == 0 && in.fwd_warps == 0 && in.bwd_batch == 0) {
    *out = CfgsRenderSchedule{kRenderBatch, 4, 64, in.bin_launch};
    return true;
  }
  const bool fwd_ok = in.fwd_warps == 4 ? (in.fwd_batch == 64 || in.fwd_batch == 128 || in.fwd_batch == 256)
                                        : (in.fwd_warps == 8 && (in.fwd_batch == 128 || in.fwd_batch == 256));
  const bool bwd_ok = in.bwd_batch == 32 || in.bwd_batch == 64 || in.bwd_batch == 128;
  if (!fwd_ok || !bwd_ok) return false;
  *out = CfgsRenderSchedule{in.fwd_batch, in.fwd_warps, in.bwd_batch, in.bin_launch};
  return true;
}

}  // namespace cfgs

using namespace cfgs;

extern "C" int cfgs_render_schedule_check(const CfgsRenderSchedule* s, CfgsRenderSchedule* resolved) {
  if (!s) return CFGS_ERR_INVALID_ARGUMENT;
  CfgsRenderSchedule r;
  if (!resolve_schedule(*s, &r)) return CFGS_ERR_INVALID_ARGUMENT;
  if (resolved) *resolved = r;
  return CFGS_OK;
}

extern "C" int cfgs_composite_forward(const CfgsSettings* s, int32_t num_gaussians, const void* geom, const void* image,
                                      const void* binning, int64_t capacity, float* out_color, float* out_depth,
                                      float* out_alpha, void* stream) {
  if (!s || !geom || !image || !binning || !out_color || capacity < 0 || !s->bg || num_gaussians < 0)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (s->image_width <= 0 || s->image_height <= 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity > 0x7fffffffll) return CFGS_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  ImageLayout IL(s->image_width, s->image_height);
  ImageView iv(const_cast<void*>(image), s->image_width, s->image_height);
  GeomView gv(const_cast<void*>(geom), num_gaussians);
  BinningView bv(const_cast<void*>(binning), capacity);
  RenderArgs<SingleScene> ra;
  ra.scenes.d = single_scene_desc(s, num_gaussians, 0);
  ra.tile_range = iv.tile_range;
  ra.sorted_gid = bv.sorted_gid;
  ra.xy = gv.xy;
  ra.conic_op = gv.conic_op;
  ra.rgbd = gv.rgbd;
  ra.final_T = iv.final_T;
  ra.n_contrib = iv.n_contrib;
  ra.out_color = out_color;
  ra.out_depth = out_depth;
  ra.out_alpha = out_alpha;
  ra.cap = capacity;
  ra.counts = iv.counts;
  if (!resolve_schedule(s->schedule, &ra.sched)) return CFGS_ERR_INVALID_ARGUMENT;
  launch_render_fwd(ra, IL.num_tiles, st);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_render_forward(const CfgsSettings* s, const CfgsGaussians* g, void* geom, void* image,
                                   void* binning, int64_t capacity, float* out_color, float* out_depth,
                                   float* out_alpha, void* stream) {
  int st = cfgs_bin_forward(s, g, geom, image, binning, capacity, stream);
  if (st != CFGS_OK) return st;
  return cfgs_composite_forward(s, g->num_gaussians, geom, image, binning, capacity, out_color, out_depth, out_alpha,
                                stream);
}
