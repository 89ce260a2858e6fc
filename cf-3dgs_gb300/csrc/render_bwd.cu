// Backward, part 1: the per-tile render backward with in-block gradient reduction,
// and the backward entry points (the per-Gaussian part is in preprocess_bwd.cu).
//
// Upstream accumulates every (pixel, Gaussian) gradient with a global atomicAdd.
// Here each tile reduces the gradients of its 256 pixels per instance inside the
// block (a transposing warp reduction, then a fixed-order sum over the 4 warps) and
// writes one 48-byte record per (Gaussian, tile) instance, at the instance's
// pre-sort index. A Gaussian's instances are contiguous in pre-sort order, so the
// preprocess backward sums its records in a fixed order: no atomics, bit-identical
// results run to run.
#include <mutex>

#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

constexpr int kBwdThreads = 128;  // 2 pixels per thread, 4 warps per 16x16 tile
constexpr int kWarps = kBwdThreads / 32;

// Sums an instance's per-lane terms over the warp. v[0..7] go through a transposing
// reduction (each step halves the values a lane carries: 4 + 2 + 1 shuffles, then two
// plain steps), after which lane L holds the total of v[L >> 2]; v[8] (and v[9] with
// depth gradients) take plain butterflies, every lane ending with the total. With GEOM
// (only v[0..4] formed, v[5..9] zero) the v[8] butterfly is skipped; the tree that sums
// v[0..4] is the same either way, so their totals are the same bits.
template <bool DEPTH, bool GEOM = false>
__device__ __forceinline__ void warp_reduce_terms(float (&v)[10], int lane) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const bool up = lane & 16;
    const float send = up ? v[k] : v[k + 4];
    const float keep = up ? v[k + 4] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool up = lane & 8;
    const float send = up ? v[k] : v[k + 2];
    const float keep = up ? v[k + 2] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  {
    const bool up = lane & 4;
    const float send = up ? v[0] : v[1];
    const float keep = up ? v[1] : v[0];
    v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
  if (!GEOM) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[8] += __shfl_xor_sync(0xffffffffu, v[8], o);
  }
  if (DEPTH) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[9] += __shfl_xor_sync(0xffffffffu, v[9], o);
  }
}

// d/dc of mean |clamp(c, 0, 1) - t| as autograd forms it.
__device__ __forceinline__ float l1_grad(float c, float t, float inv_numel) {
  float d = fminf(fmaxf(c, 0.0f), 1.0f) - t;
  float sgn = d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f);
  return (c >= 0.0f && c <= 1.0f) ? inv_numel * sgn : 0.0f;
}

// Forward results and upstream gradients of one pixel.
struct PixelBwd {
  float T_final, dC0, dC1, dC2, dD, dA_bg;  // dA_bg = dL/dalpha - bg . dL/dcolor
  uint32_t last;
};

// Loads pixel pix's forward state and upstream gradient (zeros outside the image).
template <class Scenes>
__device__ __forceinline__ void load_pixel(PixelBwd& p, const RenderBwdArgs<Scenes>& a, const SceneDesc& sd,
                                           bool inside, size_t pix) {
  const size_t HW = (size_t)sd.W * sd.H;
  const size_t gp = (size_t)sd.pix_base + pix;
  p.T_final = 1.0f;
  p.dC0 = p.dC1 = p.dC2 = p.dD = 0.f;
  float dA = 0.f;
  p.last = 0;
  if (inside) {
    p.T_final = a.final_T[gp];
    p.last = a.n_contrib[gp];
    const size_t cb = 3 * (size_t)sd.pix_base + pix;
    if (a.target) {
      p.dC0 = l1_grad(a.color[cb], a.target[cb], sd.inv_numel);
      p.dC1 = l1_grad(a.color[cb + HW], a.target[cb + HW], sd.inv_numel);
      p.dC2 = l1_grad(a.color[cb + 2 * HW], a.target[cb + 2 * HW], sd.inv_numel);
    } else {
      p.dC0 = a.dL_dcolor[cb];
      p.dC1 = a.dL_dcolor[cb + HW];
      p.dC2 = a.dL_dcolor[cb + 2 * HW];
      if (a.dL_ddepth) p.dD = a.dL_ddepth[gp];
      if (a.dL_dalpha) dA = a.dL_dalpha[gp];
    }
  }
  p.dA_bg = dA - (__ldg(sd.bg + 0) * p.dC0 + __ldg(sd.bg + 1) * p.dC1 + __ldg(sd.bg + 2) * p.dC2);
}

// Back-to-front state of a lane's two pixels (.x: row r, .y: row r + 4): upstream
// gradients, the transmittance being unwound, and the colour/depth accumulated behind the
// current instance (updated right after each contributing instance, which gives the
// value upstream forms from the previous instance's alpha and colour).
struct PairBwd {
  float2 T_final, dC0, dC1, dC2, dD, dA_bg;
  float2 T, acc0, acc1, acc2, accd;
  uint32_t last0, last1;
};

__device__ __forceinline__ PairBwd make_pair(const PixelBwd& p, const PixelBwd& q) {
  PairBwd P;
  P.T_final = make_float2(p.T_final, q.T_final);
  P.dC0 = make_float2(p.dC0, q.dC0);
  P.dC1 = make_float2(p.dC1, q.dC1);
  P.dC2 = make_float2(p.dC2, q.dC2);
  P.dD = make_float2(p.dD, q.dD);
  P.dA_bg = make_float2(p.dA_bg, q.dA_bg);
  P.T = P.T_final;
  P.acc0 = P.acc1 = P.acc2 = P.accd = make_float2(0.f, 0.f);
  P.last0 = p.last;
  P.last1 = q.last;
  return P;
}

// Unwinds one instance at list position c for both pixels and adds their terms to v:
// with g = G dL/dalpha (G the Gaussian's value at the pixel, d = mean - pixel),
// v0..v4 += g (dx, dy, dx^2, dx dy, dy^2), v5 += g, v6..v8 += w dL/drgb, v9 += w
// dL/ddepth (w = alpha T). The per-instance factors (opacity, conic) are applied after
// the reduction (finish_record). A pixel the instance did not reach in the forward pass
// keeps its state: its factors are 1 (transmittance) and 0 (alpha, G). Returns whether
// the instance contributed to either pixel. With GEOM only v0..v4 are formed (the terms
// of dL/dmean2D and dL/dconic; v5..v8 stay zero), with the same operations.
template <bool DEPTH, bool GEOM = false>
__device__ __forceinline__ bool unwind_pair(PairBwd& P, int c, float pxf, float2 pyf, const float4& m, const float4& co,
                                            const float4* s_rgbd, int j, float (&v)[10]) {
  const bool in0 = c < (int)P.last0, in1 = c < (int)P.last1;
  if (!(in0 || in1)) return false;
  const float dx = m.x - pxf;
  const float2 dy = sub2(splat2(m.y), pyf);
  const float2 power = gauss_power2(co.x, co.y, co.z, dx, dy);
  bool a0 = in0 && !(power.x > 0.0f || power.x < m.z);
  bool a1 = in1 && !(power.y > 0.0f || power.y < m.z);
  if (!(a0 || a1)) return false;
  const float2 G = exp_ref_inrange2(power);
  float2 alpha = mul2(splat2(co.w), G);
  alpha.x = fminf(CFGS_ALPHA_MAX, alpha.x);
  alpha.y = fminf(CFGS_ALPHA_MAX, alpha.y);
  a0 = a0 && !(alpha.x < CFGS_ALPHA_MIN);
  a1 = a1 && !(alpha.y < CFGS_ALPHA_MIN);
  if (!(a0 || a1)) return false;
  const float4 col = s_rgbd[j];
  const float2 om = sub2(splat2(1.0f), alpha);
  float r0, r1;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(om.x));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(om.y));
  const float2 inv = make_float2(a0 ? r0 : 1.0f, a1 ? r1 : 1.0f);
  const float2 am = make_float2(a0 ? alpha.x : 0.0f, a1 ? alpha.y : 0.0f);
  P.T = mul2(P.T, inv);
  const float2 w = mul2(am, P.T);
  if (!GEOM) {
    v[6] = fmaf(P.dC0.y, w.y, fmaf(P.dC0.x, w.x, v[6]));
    v[7] = fmaf(P.dC1.y, w.y, fmaf(P.dC1.x, w.x, v[7]));
    v[8] = fmaf(P.dC2.y, w.y, fmaf(P.dC2.x, w.x, v[8]));
  }
  const float2 e0 = sub2(splat2(col.x), P.acc0), e1 = sub2(splat2(col.y), P.acc1), e2 = sub2(splat2(col.z), P.acc2);
  float2 dLda = mul2(e0, P.dC0);
  dLda = fma2(e1, P.dC1, dLda);
  dLda = fma2(e2, P.dC2, dLda);
  P.acc0 = fma2(am, e0, P.acc0);
  P.acc1 = fma2(am, e1, P.acc1);
  P.acc2 = fma2(am, e2, P.acc2);
  if (DEPTH) {
    v[9] = fmaf(P.dD.y, w.y, fmaf(P.dD.x, w.x, v[9]));
    const float2 ed = sub2(splat2(col.w), P.accd);
    dLda = fma2(ed, P.dD, dLda);
    P.accd = fma2(am, ed, P.accd);
  }
  dLda = mul2(dLda, P.T);
  dLda = fma2(mul2(P.T_final, inv), P.dA_bg, dLda);
  const float2 g = mul2(make_float2(a0 ? G.x : 0.0f, a1 ? G.y : 0.0f), dLda);  // d/d opacity
  const float sg = g.x + g.y;
  if (!GEOM) v[5] += sg;
  const float sx = sg * dx;  // both pixels share dx
  const float2 gy = mul2(g, dy);
  v[0] += sx;
  v[1] += gy.x + gy.y;
  v[2] = fmaf(sx, dx, v[2]);
  v[3] = fmaf(g.y * dx, dy.y, fmaf(g.x * dx, dy.x, v[3]));
  v[4] = fmaf(gy.y, dy.y, fmaf(gy.x, dy.x, v[4]));
  return true;
}

// Record of one instance from its summed terms s (unwind_step) and its (ca, cb, cc,
// opacity): power = ca dx^2 + cb dx dy + cc dy^2 with ca = -A/2, cb = -B, cc = -C/2 for
// the conic (A, B, C), so dL/dpower = opacity g and
//   dL/dmean2D = opacity (2 ca Sx + cb Sy, 2 cc Sy + cb Sx),
//   dL/d(A, B, C) = -opacity (Sxx / 2, Sxy, Syy / 2).
__device__ __forceinline__ void finish_record(float4* rec, const float (&s)[10], const float4& co) {
  const float op = co.w;
  const float dmx = op * fmaf(2.f * co.x, s[0], co.y * s[1]);
  const float dmy = op * fmaf(2.f * co.z, s[1], co.y * s[0]);
  rec[0] = make_float4(dmx, dmy, -0.5f * op * s[2], -op * s[3]);
  rec[1] = make_float4(-0.5f * op * s[4], s[5], s[6], s[7]);
  rec[2] = make_float4(s[8], s[9], 0.f, 0.f);
}

// One block of 128 threads per tile with the forward's pixel boxes (warp w: 8x8 box,
// lane: rows r and r + 4) and exact shortcuts (box_may_contribute per warp and
// instance, alpha_threshold per pixel). A lane adds its two pixels' terms before the
// warp reduction; the cross-warp sum of an instance adds only the warps that kept it
// (the others' terms are exact zeros). BATCH instances are staged per round; the
// records do not depend on it (each instance's sums are formed the same way whatever
// batch it is staged in), so the batch is a schedule choice.
template <class Scenes, bool DEPTH, int BATCH, bool GEOM = false>
__global__ void __launch_bounds__(kBwdThreads, 7) k_render_bwd(RenderBwdArgs<Scenes> a) {
  static_assert(BATCH % 32 == 0 && BATCH <= kBwdThreads, "whole ballot words, one staged instance per thread");
  constexpr int kBwdBatch = BATCH;
  // Staging buffers come in pairs: batch b - 1 is copied asynchronously (cp.async; its
  // Gaussian ids were loaded a batch earlier) while batch b is unwound; two block
  // barriers per batch (staged, then partial sums complete).
  __shared__ float4 s_xyt[2][kBwdBatch];
  __shared__ float4 s_co[2][kBwdBatch];
  __shared__ float4 s_rgbd[2][kBwdBatch];
  __shared__ uint32_t s_pidx[2][kBwdBatch];
  __shared__ float s_part[kWarps][kBwdBatch][10];
  __shared__ uint32_t s_keep[kWarps][kBwdBatch / 32];
  __shared__ uint32_t s_max;
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const int tile = blockIdx.x;
  const SceneDesc& sd = a.scenes.for_tile(tile);
  const int lt = tile - sd.tile_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bx0 = (lt % sd.grid_x) * kTileX + (warp & 1) * 8;
  const int by0 = (lt / sd.grid_x) * kTileY + (warp >> 1) * 8;
  const int px = bx0 + (lane & 7), py0 = by0 + (lane >> 3), py1 = py0 + 4;
  const float bxf0 = (float)bx0, bxf1 = (float)(bx0 + 7), byf0 = (float)by0, byf1 = (float)(by0 + 7);
  const bool in0 = px < sd.W && py0 < sd.H, in1 = px < sd.W && py1 < sd.H;
  const float pxf = (float)px, pyf0 = (float)py0, pyf1 = (float)py1;
  const uint32_t lo = a.tile_range[tile];
  const int n = (int)(a.tile_range[tile + 1] - lo);

  PixelBwd p0, p1;
  load_pixel(p0, a, sd, in0, in0 ? (size_t)py0 * sd.W + px : 0);
  load_pixel(p1, a, sd, in1, in1 ? (size_t)py1 * sd.W + px : 0);
  PairBwd pp = make_pair(p0, p1);
  const float2 pyf = make_float2(pyf0, pyf1);
  if (threadIdx.x == 0) s_max = 0;
  __syncthreads();
  const uint32_t my_last = max(p0.last, p1.last);
  if (my_last) atomicMax(&s_max, my_last);
  // instances at or past the warp's largest contributor count reach none of its pixels
  const int warp_last = (int)__reduce_max_sync(0xffffffffu, my_last);
  __syncthreads();
  const int max_last = (int)s_max;

  const int t = threadIdx.x;
  auto count_of = [&](int b) { return min(kBwdBatch, max_last - b * kBwdBatch); };
  uint32_t gnext = 0;
  auto load_id = [&](int b) { gnext = t < count_of(b) ? a.sorted_gid[lo + b * kBwdBatch + t] : 0u; };
  auto issue = [&](int b, int buf) {
    if (t < count_of(b)) {
      const uint32_t i = lo + (uint32_t)(b * kBwdBatch + t);
      cp_async4(&s_pidx[buf][t], a.sorted_pidx + i);
      cp_async8(&s_xyt[buf][t], a.xy + gnext);
      cp_async16(&s_co[buf][t], a.conic_op + gnext);
      cp_async16(&s_rgbd[buf][t], a.rgbd + gnext);
    }
    cp_async_commit();
  };
  const int nb = (max_last + kBwdBatch - 1) / kBwdBatch;
  if (nb > 0) {
    load_id(nb - 1);
    issue(nb - 1, 0);
    if (nb > 1) load_id(nb - 2);
  }
  for (int k = 0; k < nb; ++k) {
    const int b = nb - 1 - k, cur = k & 1;
    const int base = b * kBwdBatch;
    const int cnt = count_of(b);
    cp_async_wait_all();
    if (t < cnt) {  // raw (x, y) and conic -> render form, own slot
      const float4 co = s_co[cur][t];
      s_xyt[cur][t].z = alpha_threshold(co.w);
      s_co[cur][t] = make_float4(-0.5f * co.x, -co.y, -0.5f * co.z, co.w);
    }
    __syncthreads();  // batch b staged; batch b + 1 finished, so its buffers are free
    if (b > 0) {
      issue(b - 1, cur ^ 1);
      if (b > 1) load_id(b - 2);
    }
    const float4* s_xyt_b = s_xyt[cur];
    const float4* s_co_b = s_co[cur];
    const float4* s_rgbd_b = s_rgbd[cur];
    uint32_t keep[kBwdBatch / 32];
#pragma unroll
    for (int r = 0; r < kBwdBatch / 32; ++r) {
      const int j = r * 32 + lane;
      bool kp = false;
      if (j < cnt && base + j < warp_last) {
        const float4 xyt = s_xyt_b[j];
        const float4 co = s_co_b[j];
        kp = box_may_contribute(make_float2(xyt.x, xyt.y), co.x, co.y, co.z, xyt.z, bxf0, bxf1, byf0, byf1);
      }
      keep[r] = __ballot_sync(0xffffffffu, kp);
      if (lane == 0) s_keep[warp][r] = keep[r];
    }
#pragma unroll
    for (int r = kBwdBatch / 32 - 1; r >= 0; --r) {
      uint32_t mk = keep[r];
      while (mk) {
        const int bit = 31 - __clz(mk);
        mk &= ~(1u << bit);
        const int j = r * 32 + bit;
        const int c = base + j;
        float v[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) v[q] = 0.f;
        const float4 m = s_xyt_b[j];
        const float4 co = s_co_b[j];
        const bool contrib = unwind_pair<DEPTH, GEOM>(pp, c, pxf, pyf, m, co, s_rgbd_b, j, v);
        if (__ballot_sync(0xffffffffu, contrib)) {
          warp_reduce_terms<DEPTH, GEOM>(v, lane);
          if ((lane & 3) == 0) s_part[warp][j][lane >> 2] = v[0];
          if (lane == 0) {
            s_part[warp][j][8] = v[8];
            s_part[warp][j][9] = v[9];
          }
        } else if (lane < 10) {
          s_part[warp][j][lane] = 0.f;
        }
      }
    }
    __syncthreads();  // every warp's partial sums of batch b are in
    if (t < cnt) {
      const int j = t;
      float sum[10];
#pragma unroll
      for (int q = 0; q < 10; ++q) sum[q] = 0.f;
      bool kept = false;
#pragma unroll
      for (int w = 0; w < kWarps; ++w)
        if ((s_keep[w][j >> 5] >> (j & 31)) & 1u) {
          kept = true;
#pragma unroll
          for (int q = 0; q < 10; ++q) sum[q] += s_part[w][j][q];
        }
      // An instance no warp kept has exact-zero gradients: no record, its byte stays 0.
      if (kept) {
        const uint32_t pidx = s_pidx[cur][j];
        finish_record(a.records + (size_t)kRecordFloat4 * pidx, sum, s_co_b[j]);
        a.written[pidx] = 1;
      }
    }
  }
  // Instances at or past the tile's last contributor reach no pixel: nothing to write.
}

template <class Scenes, bool DEPTH, bool GEOM = false>
void launch_render_bwd_depth(const RenderBwdArgs<Scenes>& a, int tiles, int batch, cudaStream_t st) {
  if (batch == 32) k_render_bwd<Scenes, DEPTH, 32, GEOM><<<tiles, kBwdThreads, 0, st>>>(a);
  else if (batch == 128) k_render_bwd<Scenes, DEPTH, 128, GEOM><<<tiles, kBwdThreads, 0, st>>>(a);
  else k_render_bwd<Scenes, DEPTH, 64, GEOM><<<tiles, kBwdThreads, 0, st>>>(a);
}

template <class Scenes>
void launch_render_bwd(const RenderBwdArgs<Scenes>& a, int tiles, cudaStream_t st) {
  const int batch = a.sched.bwd_batch;
  if constexpr (Scenes::kBatched) {  // batched solves never ask for depth gradients
    if (a.geom_only) launch_render_bwd_depth<Scenes, false, true>(a, tiles, batch, st);
    else launch_render_bwd_depth<Scenes, false>(a, tiles, batch, st);
  } else {
    if (a.dL_ddepth) launch_render_bwd_depth<Scenes, true>(a, tiles, batch, st);
    else launch_render_bwd_depth<Scenes, false>(a, tiles, batch, st);
  }
}
template void launch_render_bwd<SingleScene>(const RenderBwdArgs<SingleScene>&, int, cudaStream_t);
template void launch_render_bwd<SceneTable>(const RenderBwdArgs<SceneTable>&, int, cudaStream_t);

}  // namespace cfgs

using namespace cfgs;

extern "C" int cfgs_render_backward(const CfgsSettings* s, int32_t num_gaussians, const void* geom, const void* image,
                                    const void* binning, int64_t capacity, void* scratch, const float* dL_dcolor,
                                    const float* dL_ddepth, const float* dL_dalpha, void* stream) {
  if (!s || !geom || !image || !binning || !scratch || !dL_dcolor || !s->bg || num_gaussians < 0)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (s->image_width <= 0 || s->image_height <= 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity < 0 || capacity > 0x7fffffffll) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  ImageLayout IL(s->image_width, s->image_height);
  ImageView iv(const_cast<void*>(image), s->image_width, s->image_height);
  GeomView gv(const_cast<void*>(geom), num_gaussians);
  BinningView bv(const_cast<void*>(binning), capacity);
  RenderBwdArgs<SingleScene> ra;
  ra.scenes.d = single_scene_desc(s, num_gaussians, 0);
  ra.tile_range = iv.tile_range;
  ra.sorted_gid = bv.sorted_gid;
  ra.sorted_pidx = bv.sorted_pidx;
  ra.xy = gv.xy;
  ra.conic_op = gv.conic_op;
  ra.rgbd = gv.rgbd;
  ra.final_T = iv.final_T;
  ra.n_contrib = iv.n_contrib;
  ra.dL_dcolor = dL_dcolor;
  ra.dL_ddepth = dL_ddepth;
  ra.dL_dalpha = dL_dalpha;
  ra.color = nullptr;
  ra.target = nullptr;
  const ScratchLayout SL(capacity);
  ra.records = reinterpret_cast<float4*>(static_cast<char*>(scratch) + SL.records);
  ra.written = reinterpret_cast<uint8_t*>(static_cast<char*>(scratch) + SL.written);
  ra.cap = capacity;
  ra.counts = iv.counts;
  if (!resolve_schedule(s->schedule, &ra.sched)) return CFGS_ERR_INVALID_ARGUMENT;
  ra.geom_only = false;
  if (capacity > 0 && cudaMemsetAsync(ra.written, 0, (size_t)capacity, st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  launch_render_bwd(ra, IL.num_tiles, st);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_preprocess_backward(const CfgsSettings* s, const CfgsGaussians* g, const int32_t* radii,
                                        const void* geom, const void* image, int64_t capacity, const void* scratch,
                                        const CfgsGradients* out, void* stream) {
  if (!s || !g || !geom || !image || !scratch || !out || !s->viewmatrix || !s->projmatrix)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (g->num_gaussians == 0) return CFGS_OK;
  if (g->num_gaussians < 0 || !radii || !g->means3D || !g->opacities) return CFGS_ERR_INVALID_ARGUMENT;
  if (!out->dL_dmeans2D || !out->dL_dcolors || !out->dL_dopacity || !out->dL_dmeans3D || !out->dL_dcov3D)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (!g->cov3D_precomp && (!out->dL_dscales || !out->dL_drotations || !g->scales || !g->rotations))
    return CFGS_ERR_INVALID_ARGUMENT;
  if ((g->shs == nullptr) == (g->colors_precomp == nullptr)) return CFGS_ERR_INVALID_ARGUMENT;
  if (g->shs && !s->campos) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity < 0 || capacity > 0x7fffffffll) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  ImageView iv(const_cast<void*>(image), s->image_width, s->image_height);
  PreBwdArgs<SingleScene> pa;
  pa.scenes.d = single_scene_desc(s, g->num_gaussians, g->sh_coeffs);
  pa.g = *g;
  pa.radii = radii;
  pa.geom = GeomView(const_cast<void*>(geom), g->num_gaussians);
  const ScratchLayout SL(capacity);
  pa.records = reinterpret_cast<const float4*>(static_cast<const char*>(scratch) + SL.records);
  pa.written = reinterpret_cast<const uint8_t*>(static_cast<const char*>(scratch) + SL.written);
  pa.out = *out;
  pa.total_slots = g->num_gaussians;
  pa.cap = capacity;
  pa.counts = iv.counts;
  pa.pose_partials = nullptr;
  pa.flags = &iv.counts->flags;
  pa.sh_bulk = g->shs != nullptr && g->sh_coeffs == CFGS_SH_BULK_COEFFS && (((uintptr_t)g->shs) & 15) == 0 &&
               (out->dL_dsh == nullptr || (((uintptr_t)out->dL_dsh) & 15) == 0);
  launch_preprocess_bwd(pa, div_up(g->num_gaussians, 256), st);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_backward(const CfgsSettings* s, const CfgsGaussians* g, const int32_t* radii, const void* geom,
                             const void* image, const void* binning, int64_t capacity, void* scratch,
                             const float* dL_dcolor, const float* dL_ddepth, const float* dL_dalpha,
                             const CfgsGradients* out, void* stream) {
  if (!g) return CFGS_ERR_INVALID_ARGUMENT;
  if (g->num_gaussians == 0) return CFGS_OK;
  int st = cfgs_render_backward(s, g->num_gaussians, geom, image, binning, capacity, scratch, dL_dcolor, dL_ddepth,
                                dL_dalpha, stream);
  if (st != CFGS_OK) return st;
  return cfgs_preprocess_backward(s, g, radii, geom, image, capacity, scratch, out, stream);
}

// ---- allocation-free backward ----------------------------------------------------
// Some callers cannot allocate device memory when they call the rasteriser: plugin
// hosts that hand a plugin only its input and output buffers, and services that must
// not allocate once they are serving. This entry point runs the same two kernels as
// cfgs_backward, but its per-instance scratch (gradient records and their written
// bytes, the layout cfgs_backward_scratch_bytes sizes) lives in the fixed array below
// instead of a caller-provided buffer. Every GPU that loads this library holds the
// array (30.6 MiB) until the process exits.
constexpr size_t kNoallocRecordBytes = ((size_t)CFGS_NOALLOC_MAX_INSTANCES * 16 * kRecordFloat4 + 255) & ~size_t(255);
constexpr size_t kNoallocScratchBytes = kNoallocRecordBytes + (((size_t)CFGS_NOALLOC_MAX_INSTANCES + 255) & ~size_t(255));
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

namespace {
// The array's device address belongs to the CUDA context that loaded this library's
// device code: after cudaDeviceReset, or in another context on the same device, the
// module is loaded again and the array may sit elsewhere. So the address is cached per
// context, keyed by the driver's context id (unique for the life of the process, even
// when a new context reuses a freed one's handle), and looked up again for a context
// not seen before. The driver functions come through the runtime's entry-point query,
// so the library does not link the driver library itself.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
constexpr int kNoallocCacheSize = 64;
struct NoallocEntry {
  unsigned long long ctx_id;
  void* ptr;
};
std::mutex g_noalloc_mutex;
NoallocEntry g_noalloc_cache[kNoallocCacheSize];
int g_noalloc_used = 0, g_noalloc_next = 0;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

bool context_id(unsigned long long* id) {
  void* ctx = nullptr;
  if (g_ctx_get_current(&ctx) != 0 || ctx == nullptr) return false;
  return g_ctx_get_id(ctx, id) == 0;
}

// Device address of g_noalloc_scratch in the current context. The host-side name of
// the array is only a stand-in for it, so the address comes from cudaGetSymbolAddress,
// called with the caller's device current, once per context.
int noalloc_scratch(void** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&g_ctx_get_current), 12000,
                                         cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", reinterpret_cast<void**>(&g_ctx_get_id), 12000,
                                         cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess) {
      g_ctx_get_current = nullptr;
      g_ctx_get_id = nullptr;
      return CFGS_ERR_LAUNCH;
    }
  }
  unsigned long long id = 0;
  const bool have_ctx = context_id(&id);
  if (have_ctx)
    for (int i = 0; i < g_noalloc_used; ++i)
      if (g_noalloc_cache[i].ctx_id == id) {
        *out = g_noalloc_cache[i].ptr;
        return CFGS_OK;
      }
  // Not seen yet (or no context current: the lookup below makes the device's primary
  // context current and loads the module).
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return CFGS_ERR_LAUNCH;
  if (!context_id(&id)) return CFGS_ERR_LAUNCH;
  const int slot = g_noalloc_used < kNoallocCacheSize ? g_noalloc_used++ : (g_noalloc_next++ % kNoallocCacheSize);
  g_noalloc_cache[slot] = NoallocEntry{id, p};
  *out = p;
  return CFGS_OK;
}
}  // namespace

extern "C" int cfgs_backward_noalloc(const CfgsSettings* s, const CfgsGaussians* g, const int32_t* radii,
                                     const void* geom, const void* image, const void* binning, int64_t capacity,
                                     const float* dL_dcolor, const float* dL_ddepth, const float* dL_dalpha,
                                     const CfgsGradients* out, void* stream) {
  if (capacity < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity > CFGS_NOALLOC_MAX_INSTANCES) return CFGS_ERR_TOO_LARGE;
  void* scratch = nullptr;
  int st = noalloc_scratch(&scratch);
  if (st != CFGS_OK) return st;
  return cfgs_backward(s, g, radii, geom, image, binning, capacity, scratch, dL_dcolor, dL_ddepth, dL_dalpha, out,
                       stream);
}
