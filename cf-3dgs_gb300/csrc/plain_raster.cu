// The plain GPU path: the published 3D Gaussian Splatting rasteriser's structure
// (64-bit keys and one radix sort, one thread per pixel, global atomic gradients), the
// GPU comparison point for the tuned kernels. The per-pixel arithmetic is shared with
// them (gauss_power, exp_ref, the same operation order; this file is compiled without
// FMA contraction like render_fwd.cu), so the forward agrees bit for bit and the timing
// difference is the structure alone.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "cfgs_plain.h"
#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {
namespace {

constexpr int kPlainThreads = kTilePixels;  // one thread per pixel of a 16x16 tile

// Workspace: scan offsets, the key/id buffers the sort reads and writes, per-tile
// ranges, per-Gaussian gradient accumulators (one 48-byte record per Gaussian, the
// layout the per-Gaussian backward reads), the identity views that let that kernel read
// one record per Gaussian, and the sort's temporary storage.
struct PlainLayout {
  size_t offsets, keys_in, keys_out, vals_in, vals_out, ranges, acc, iota, ones, marks, temp, total;
  size_t temp_bytes;
  PlainLayout(int32_t n, int64_t cap, int tiles, size_t temp_b) : temp_bytes(temp_b) {
    const size_t N = (size_t)(n > 0 ? n : 1), K = (size_t)(cap > 0 ? cap : 1), T = (size_t)(tiles > 0 ? tiles : 1);
    size_t o = 0;
    offsets = o;  o = align256(o + sizeof(uint32_t) * N);
    keys_in = o;  o = align256(o + sizeof(uint64_t) * K);
    keys_out = o; o = align256(o + sizeof(uint64_t) * K);
    vals_in = o;  o = align256(o + sizeof(uint32_t) * K);
    vals_out = o; o = align256(o + sizeof(uint32_t) * K);
    ranges = o;   o = align256(o + sizeof(uint2) * T);
    acc = o;      o = align256(o + sizeof(float4) * kRecordFloat4 * N);
    iota = o;     o = align256(o + sizeof(uint32_t) * N);
    ones = o;     o = align256(o + sizeof(uint32_t) * N);
    marks = o;    o = align256(o + N);
    temp = o;     o = align256(o + temp_bytes);
    total = o;
  }
};

// Temporary storage of the scan over N and of the sort over `cap` 64-bit keys (queried
// for all 64 key bits, the most any call sorts). 0 on a failed query.
size_t plain_temp_bytes(int32_t n, int64_t cap) {
  size_t scan_b = 0, sort_b = 0;
  const int nn = n > 0 ? n : 1, kk = (int)(cap > 0 ? cap : 1);
  if (cub::DeviceScan::InclusiveSum(nullptr, scan_b, (const uint32_t*)nullptr, (uint32_t*)nullptr, nn) != cudaSuccess)
    return 0;
  if (cub::DeviceRadixSort::SortPairs(nullptr, sort_b, (const uint64_t*)nullptr, (uint64_t*)nullptr,
                                      (const uint32_t*)nullptr, (uint32_t*)nullptr, kk, 0, 64) != cudaSuccess)
    return 0;
  return scan_b > sort_b ? scan_b : sort_b;
}

// One thread per Gaussian: its instances' keys (tile index << 32 | depth bits) and ids
// from its first slot (inclusive scan - own count), tiles row by row over its
// rectangle; also the identity views of the per-Gaussian backward.
__global__ void k_plain_duplicate(int32_t n, int grid_x, const uint32_t* touched, const uint32_t* offsets,
                                  const uint2* rect, const float4* rgbd, uint64_t* keys, uint32_t* vals,
                                  uint32_t* iota, uint32_t* ones, uint8_t* marks) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  iota[g] = (uint32_t)g;
  ones[g] = 1u;
  marks[g] = 1u;
  const uint32_t nt = touched[g];
  if (nt == 0) return;
  uint32_t o = offsets[g] - nt;
  const uint2 r = rect[g];
  const uint32_t x0 = r.x & 0xffffu, y0 = r.x >> 16, x1 = r.y & 0xffffu, y1 = r.y >> 16;
  const uint64_t d = (uint64_t)__float_as_uint(rgbd[g].w);
  for (uint32_t y = y0; y < y1; ++y)
    for (uint32_t x = x0; x < x1; ++x, ++o) {
      keys[o] = ((uint64_t)(y * (uint32_t)grid_x + x) << 32) | d;
      vals[o] = (uint32_t)g;
    }
}

// One thread per sorted instance: where the tile index changes, one range ends and the
// next begins (ranges are zeroed beforehand: tiles without instances stay empty).
__global__ void k_plain_ranges(int64_t K, const uint64_t* keys, uint2* ranges) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  const uint32_t t = (uint32_t)(keys[i] >> 32);
  if (i == 0) {
    ranges[t].x = 0;
  } else {
    const uint32_t p = (uint32_t)(keys[i - 1] >> 32);
    if (p != t) {
      ranges[p].y = (uint32_t)i;
      ranges[t].x = (uint32_t)i;
    }
  }
  if (i == K - 1) ranges[t].y = (uint32_t)K;
}

struct PlainFwdArgs {
  SceneDesc sd;
  const uint2* ranges;
  const uint32_t* ids;
  const float2* xy;
  const float4* conic_op;
  const float4* rgbd;
  float* final_T;
  uint32_t* n_contrib;
  float* out_color;
  float* out_depth;
  float* out_alpha;
};

// Front to back, one thread per pixel; the block fetches 256 instances per round into
// shared memory and stops when every pixel of the tile is saturated (transmittance
// below 1e-4) or the tile's list ends.
__global__ void __launch_bounds__(kPlainThreads) k_plain_render_fwd(PlainFwdArgs a) {
  __shared__ uint32_t s_id[kPlainThreads];
  __shared__ float2 s_xy[kPlainThreads];
  __shared__ float4 s_co[kPlainThreads];
  const SceneDesc& sd = a.sd;
  const int tile = blockIdx.x;
  const int t = threadIdx.x;
  const int px = (tile % sd.grid_x) * kTileX + (t % kTileX), py = (tile / sd.grid_x) * kTileY + (t / kTileX);
  const bool inside = px < sd.W && py < sd.H;
  const float pxf = (float)px, pyf = (float)py;
  const uint2 rg = a.ranges[tile];
  const int n = (int)(rg.y - rg.x);
  bool done = !inside;
  float T = 1.0f, C0 = 0.f, C1 = 0.f, C2 = 0.f, D = 0.f;
  uint32_t contributor = 0, last = 0;
  for (int base = 0; base < n; base += kPlainThreads) {
    if (__syncthreads_count(done) == kPlainThreads) break;
    if (base + t < n) {
      const uint32_t g = a.ids[rg.x + base + t];
      s_id[t] = g;
      s_xy[t] = a.xy[g];
      s_co[t] = a.conic_op[g];
    }
    __syncthreads();
    const int cnt = min(kPlainThreads, n - base);
    for (int j = 0; !done && j < cnt; ++j) {
      ++contributor;
      const float4 co = s_co[j];
      const float dx = s_xy[j].x - pxf, dy = s_xy[j].y - pyf;
      const float power = gauss_power(-0.5f * co.x, -co.y, -0.5f * co.z, dx, dy);
      if (power > 0.0f) continue;
      const float alpha = fminf(CFGS_ALPHA_MAX, co.w * exp_ref(power));
      if (alpha < CFGS_ALPHA_MIN) continue;
      const float test_T = T * (1.0f - alpha);
      if (test_T < CFGS_T_MIN) {
        done = true;
        continue;
      }
      const float4 f = a.rgbd[s_id[j]];
      const float w = alpha * T;
      C0 = fmaf(f.x, w, C0);
      C1 = fmaf(f.y, w, C1);
      C2 = fmaf(f.z, w, C2);
      D = fmaf(f.w, w, D);
      T = test_T;
      last = contributor;
    }
  }
  if (inside) {
    const size_t HW = (size_t)sd.W * sd.H, pix = (size_t)py * sd.W + px;
    a.final_T[pix] = T;
    a.n_contrib[pix] = last;
    a.out_color[pix] = fmaf(T, sd.bg[0], C0);
    a.out_color[HW + pix] = fmaf(T, sd.bg[1], C1);
    a.out_color[2 * HW + pix] = fmaf(T, sd.bg[2], C2);
    if (a.out_depth) a.out_depth[pix] = D;
    if (a.out_alpha) a.out_alpha[pix] = 1.0f - T;
  }
}

struct PlainBwdArgs {
  SceneDesc sd;
  const uint2* ranges;
  const uint32_t* ids;
  const float2* xy;
  const float4* conic_op;
  const float4* rgbd;
  const float* final_T;
  const uint32_t* n_contrib;
  const float* dL_dcolor;
  const float* dL_ddepth;
  const float* dL_dalpha;
  float* acc;  // [N][12]: dmean2D (2, pixels), dconic (3), dopacity, drgb (3), ddepth, -, -
};

// Back to front, one thread per pixel, rounds of 256 instances fetched from the end of
// the tile's list. Each contribution re-forms alpha as the forward did, unwinds the
// transmittance, rebuilds the colour behind it and adds its terms to the Gaussian's
// accumulators with one atomic add per term.
__global__ void __launch_bounds__(kPlainThreads) k_plain_render_bwd(PlainBwdArgs a) {
  __shared__ uint32_t s_id[kPlainThreads];
  __shared__ float2 s_xy[kPlainThreads];
  __shared__ float4 s_co[kPlainThreads];
  __shared__ float4 s_col[kPlainThreads];
  const SceneDesc& sd = a.sd;
  const int tile = blockIdx.x;
  const int t = threadIdx.x;
  const int px = (tile % sd.grid_x) * kTileX + (t % kTileX), py = (tile / sd.grid_x) * kTileY + (t / kTileX);
  const bool inside = px < sd.W && py < sd.H;
  const float pxf = (float)px, pyf = (float)py;
  const uint2 rg = a.ranges[tile];
  const int n = (int)(rg.y - rg.x);
  const size_t HW = (size_t)sd.W * sd.H, pix = inside ? (size_t)py * sd.W + px : 0;
  const float T_final = inside ? a.final_T[pix] : 0.0f;
  const uint32_t last = inside ? a.n_contrib[pix] : 0u;
  float dC[3] = {0.f, 0.f, 0.f}, dD = 0.f, dA = 0.f;
  if (inside) {
    dC[0] = a.dL_dcolor[pix];
    dC[1] = a.dL_dcolor[HW + pix];
    dC[2] = a.dL_dcolor[2 * HW + pix];
    if (a.dL_ddepth) dD = a.dL_ddepth[pix];
    if (a.dL_dalpha) dA = a.dL_dalpha[pix];
  }
  const float bg_dot = sd.bg[0] * dC[0] + sd.bg[1] * dC[1] + sd.bg[2] * dC[2];
  const bool want_depth = a.dL_ddepth != nullptr;
  float T = T_final;
  float accum[4] = {0.f, 0.f, 0.f, 0.f}, last_col[4] = {0.f, 0.f, 0.f, 0.f}, last_alpha = 0.f;
  uint32_t contributor = (uint32_t)n;
  for (int base = 0; base < n; base += kPlainThreads) {
    __syncthreads();  // the previous round's instances are no longer read
    if (base + t < n) {
      const uint32_t g = a.ids[rg.y - 1 - (uint32_t)(base + t)];
      s_id[t] = g;
      s_xy[t] = a.xy[g];
      s_co[t] = a.conic_op[g];
      s_col[t] = a.rgbd[g];
    }
    __syncthreads();
    const int cnt = min(kPlainThreads, n - base);
    for (int j = 0; inside && j < cnt; ++j) {
      --contributor;
      if (contributor >= last) continue;
      const float4 co = s_co[j];
      const float ca = -0.5f * co.x, cb = -co.y, cc = -0.5f * co.z, op = co.w;
      const float dx = s_xy[j].x - pxf, dy = s_xy[j].y - pyf;
      const float power = gauss_power(ca, cb, cc, dx, dy);
      if (power > 0.0f) continue;
      const float G = exp_ref(power);
      const float alpha = fminf(CFGS_ALPHA_MAX, op * G);
      if (alpha < CFGS_ALPHA_MIN) continue;
      T = T / (1.0f - alpha);
      const float w = alpha * T;
      const float4 col4 = s_col[j];
      const float col[4] = {col4.x, col4.y, col4.z, col4.w};
      const float up[4] = {dC[0], dC[1], dC[2], dD};
      float dLda = 0.0f;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        accum[ch] = fmaf(last_alpha, last_col[ch], (1.0f - last_alpha) * accum[ch]);
        last_col[ch] = col[ch];
        dLda = fmaf(col[ch] - accum[ch], up[ch], dLda);
      }
      dLda *= T;
      last_alpha = alpha;
      dLda = fmaf(T_final / (1.0f - alpha), dA - bg_dot, dLda);
      const float g = G * dLda;  // dL/dopacity of this contribution
      const float dp = op * g;   // dL/dpower
      float* acc = a.acc + (size_t)s_id[j] * 12;
      atomicAdd(acc + 0, dp * fmaf(2.0f * ca, dx, cb * dy));
      atomicAdd(acc + 1, dp * fmaf(2.0f * cc, dy, cb * dx));
      atomicAdd(acc + 2, -0.5f * dx * dx * dp);
      atomicAdd(acc + 3, -dx * dy * dp);
      atomicAdd(acc + 4, -0.5f * dy * dy * dp);
      atomicAdd(acc + 5, g);
      atomicAdd(acc + 6, dC[0] * w);
      atomicAdd(acc + 7, dC[1] * w);
      atomicAdd(acc + 8, dC[2] * w);
      if (want_depth) atomicAdd(acc + 9, dD * w);
    }
  }
}

}  // namespace
}  // namespace cfgs

using namespace cfgs;

extern "C" size_t cfgs_plain_work_bytes(int32_t num_gaussians, int64_t capacity, int32_t width, int32_t height) {
  if (num_gaussians < 0 || capacity < 0 || capacity > 0x7fffffffll || width <= 0 || height <= 0) return 0;
  const size_t temp = plain_temp_bytes(num_gaussians, capacity);
  if (temp == 0) return 0;
  ImageLayout IL(width, height);
  return PlainLayout(num_gaussians, capacity, IL.num_tiles, temp).total;
}

extern "C" int cfgs_plain_bin(const CfgsSettings* s, int32_t num_gaussians, const void* geom, void* work,
                              int64_t capacity, int64_t* num_rendered, void* stream) {
  if (!s || !geom || !work || !num_rendered || num_gaussians < 0 || capacity < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (s->image_width <= 0 || s->image_height <= 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity > 0x7fffffffll) return CFGS_ERR_TOO_LARGE;
  *num_rendered = 0;
  if (num_gaussians == 0) return CFGS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t temp_b = plain_temp_bytes(num_gaussians, capacity);
  if (temp_b == 0) return CFGS_ERR_LAUNCH;
  ImageLayout IL(s->image_width, s->image_height);
  const PlainLayout L(num_gaussians, capacity, IL.num_tiles, temp_b);
  char* w = static_cast<char*>(work);
  GeomView gv(const_cast<void*>(geom), num_gaussians);
  uint32_t* offsets = reinterpret_cast<uint32_t*>(w + L.offsets);
  size_t tb = temp_b;
  if (cub::DeviceScan::InclusiveSum(w + L.temp, tb, gv.touched, offsets, num_gaussians, st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  uint32_t K = 0;
  if (cudaMemcpyAsync(&K, offsets + (num_gaussians - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  *num_rendered = K;
  if ((int64_t)K > capacity) return CFGS_ERR_CAPACITY;
  uint64_t* keys_in = reinterpret_cast<uint64_t*>(w + L.keys_in);
  uint64_t* keys_out = reinterpret_cast<uint64_t*>(w + L.keys_out);
  uint32_t* vals_in = reinterpret_cast<uint32_t*>(w + L.vals_in);
  uint32_t* vals_out = reinterpret_cast<uint32_t*>(w + L.vals_out);
  uint2* ranges = reinterpret_cast<uint2*>(w + L.ranges);
  k_plain_duplicate<<<div_up(num_gaussians, 256), 256, 0, st>>>(
      num_gaussians, IL.grid_x, gv.touched, offsets, gv.rect, gv.rgbd, keys_in, vals_in,
      reinterpret_cast<uint32_t*>(w + L.iota), reinterpret_cast<uint32_t*>(w + L.ones),
      reinterpret_cast<uint8_t*>(w + L.marks));
  CFGS_CHECK_LAUNCH(s->debug, st);
  int tile_bits = 0;
  while ((1 << tile_bits) < IL.num_tiles + 1) ++tile_bits;
  if (cudaMemsetAsync(ranges, 0, sizeof(uint2) * (size_t)IL.num_tiles, st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  if (K > 0) {
    tb = temp_b;
    if (cub::DeviceRadixSort::SortPairs(w + L.temp, tb, keys_in, keys_out, vals_in, vals_out, (int)K, 0,
                                        32 + tile_bits, st) != cudaSuccess)
      return CFGS_ERR_LAUNCH;
    k_plain_ranges<<<div_up(K, 256), 256, 0, st>>>((int64_t)K, keys_out, ranges);
    CFGS_CHECK_LAUNCH(s->debug, st);
  }
  return CFGS_OK;
}

extern "C" int cfgs_plain_render_forward(const CfgsSettings* s, int32_t num_gaussians, const void* geom, void* image,
                                         const void* work, int64_t capacity, float* out_color, float* out_depth,
                                         float* out_alpha, void* stream) {
  if (!s || !geom || !image || !work || !out_color || !s->bg || num_gaussians < 0 || capacity < 0)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (s->image_width <= 0 || s->image_height <= 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity > 0x7fffffffll) return CFGS_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t temp_b = plain_temp_bytes(num_gaussians, capacity);
  if (temp_b == 0) return CFGS_ERR_LAUNCH;
  ImageLayout IL(s->image_width, s->image_height);
  const PlainLayout L(num_gaussians, capacity, IL.num_tiles, temp_b);
  const char* w = static_cast<const char*>(work);
  ImageView iv(image, s->image_width, s->image_height);
  GeomView gv(const_cast<void*>(geom), num_gaussians);
  PlainFwdArgs a;
  a.sd = single_scene_desc(s, num_gaussians, 0);
  a.ranges = reinterpret_cast<const uint2*>(w + L.ranges);
  a.ids = reinterpret_cast<const uint32_t*>(w + L.vals_out);
  a.xy = gv.xy;
  a.conic_op = gv.conic_op;
  a.rgbd = gv.rgbd;
  a.final_T = iv.final_T;
  a.n_contrib = iv.n_contrib;
  a.out_color = out_color;
  a.out_depth = out_depth;
  a.out_alpha = out_alpha;
  if (num_gaussians == 0) {  // empty list: every tile has an empty range
    if (cudaMemsetAsync(const_cast<char*>(w) + L.ranges, 0, sizeof(uint2) * (size_t)IL.num_tiles, st) != cudaSuccess)
      return CFGS_ERR_LAUNCH;
  }
  k_plain_render_fwd<<<IL.num_tiles, kPlainThreads, 0, st>>>(a);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_plain_backward(const CfgsSettings* s, const CfgsGaussians* g, const int32_t* radii,
                                   const void* geom, const void* image, void* work, int64_t capacity,
                                   const float* dL_dcolor, const float* dL_ddepth, const float* dL_dalpha,
                                   const CfgsGradients* out, void* stream) {
  if (!s || !g || !geom || !image || !work || !out || !dL_dcolor || !s->viewmatrix || !s->projmatrix || !s->bg)
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
  if (s->image_width <= 0 || s->image_height <= 0) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  const int32_t N = g->num_gaussians;
  const size_t temp_b = plain_temp_bytes(N, capacity);
  if (temp_b == 0) return CFGS_ERR_LAUNCH;
  ImageLayout IL(s->image_width, s->image_height);
  const PlainLayout L(N, capacity, IL.num_tiles, temp_b);
  char* w = static_cast<char*>(work);
  ImageView iv(const_cast<void*>(image), s->image_width, s->image_height);
  GeomView gv(const_cast<void*>(geom), N);
  float* acc = reinterpret_cast<float*>(w + L.acc);
  if (cudaMemsetAsync(acc, 0, sizeof(float4) * kRecordFloat4 * (size_t)N, st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  PlainBwdArgs b;
  b.sd = single_scene_desc(s, N, g->sh_coeffs);
  b.ranges = reinterpret_cast<const uint2*>(w + L.ranges);
  b.ids = reinterpret_cast<const uint32_t*>(w + L.vals_out);
  b.xy = gv.xy;
  b.conic_op = gv.conic_op;
  b.rgbd = gv.rgbd;
  b.final_T = iv.final_T;
  b.n_contrib = iv.n_contrib;
  b.dL_dcolor = dL_dcolor;
  b.dL_ddepth = dL_ddepth;
  b.dL_dalpha = dL_dalpha;
  b.acc = acc;
  k_plain_render_bwd<<<IL.num_tiles, kPlainThreads, 0, st>>>(b);
  CFGS_CHECK_LAUNCH(s->debug, st);
  // The per-Gaussian backward reads instance records [offset, offset + touched) of each
  // Gaussian; here each Gaussian has exactly one, its accumulator: offset = own index,
  // touched = 1, written = 1.
  PreBwdArgs<SingleScene> pa;
  pa.scenes.d = b.sd;
  pa.g = *g;
  pa.radii = radii;
  pa.geom = gv;
  pa.geom.offset = reinterpret_cast<uint32_t*>(w + L.iota);
  pa.geom.touched = reinterpret_cast<uint32_t*>(w + L.ones);
  pa.records = reinterpret_cast<const float4*>(acc);
  pa.written = reinterpret_cast<const uint8_t*>(w + L.marks);
  pa.out = *out;
  pa.total_slots = N;
  pa.cap = capacity;
  pa.counts = iv.counts;
  pa.pose_partials = nullptr;
  pa.flags = &iv.counts->flags;
  pa.sh_bulk = g->shs != nullptr && g->sh_coeffs == CFGS_SH_BULK_COEFFS && (((uintptr_t)g->shs) & 15) == 0 &&
               (out->dL_dsh == nullptr || (((uintptr_t)out->dL_dsh) & 15) == 0);
  launch_preprocess_bwd(pa, div_up(N, 256), st);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}
