// Forward phase 2: instance emission, per-tile depth sort, tile ranges and the
// front-to-back alpha compositing of every 16x16 tile.
//
// Binning. Upstream emits K 64-bit keys (tile << 32 | depth bits) and runs one global
// stable radix sort over 32 + log2(tiles) bits. Here the tile part of the key is
// consumed by a counting sort that costs nothing extra: the preprocess already
// counted instances per tile, the scan turned the counts into tile ranges, and the
// scatter below drops each instance into its tile's range. Each tile then sorts only
// its own segment, in shared memory, by the 64-bit value (depth bits << 32 | pre-sort
// instance index). Pre-sort instance indices grow with the Gaussian index and a
// Gaussian touches a tile once, so the result is exactly the order a stable sort of
// upstream's keys gives: depth, ties broken by Gaussian index.
//
// Compiled with -fmad=false; the fmaf() calls are the only fused operations, and the
// CPU oracle performs the same sequence.
#include "cfgs_internal.cuh"

namespace cfgs {

constexpr int kSortCap = 4096;   // tile segments up to this size sort in shared memory
constexpr int kSortThreads = 256;
constexpr int kRenderBatch = 256;

__device__ __forceinline__ uint32_t block_excl_scan_256(uint32_t v, uint32_t* sh, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  uint32_t pre = 0, tot = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    uint32_t s = sh[w];
    if (w < warp) pre += s;
    tot += s;
  }
  *total = tot;
  return pre + (x - v);
}

struct ScatterArgs {
  int32_t n;
  GeomView geom;
  const uint32_t* tile_range;
  uint32_t* tile_cursor;
  int grid_x;
  BinningView bin;
  int64_t cap;
  CfgsCounts* counts;
};

// One thread per Gaussian (same 256-wide partition as the preprocess, so the block
// prefixes line up): assigns pre-sort instance indices in Gaussian order, row-major
// over the tile rectangle, and drops each instance into its tile's range.
__global__ void __launch_bounds__(kPreprocessBlock) k_scatter(ScatterArgs a) {
  __shared__ uint32_t sh[kPreprocessBlock / 32];
  if ((int64_t)a.counts->num_rendered > a.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.counts->flags, CFGS_FLAG_CAPACITY_OVERFLOW);
    return;
  }
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t t = g < a.n ? a.geom.touched[g] : 0u;
  uint32_t tot;
  uint32_t off = a.geom.block_prefix[blockIdx.x] + block_excl_scan_256(t, sh, &tot);
  if (g < a.n) a.geom.offset[g] = off;
  if (t == 0) return;
  uint2 r = a.geom.rect[g];
  int x0 = r.x & 0xffff, y0 = r.x >> 16, x1 = r.y & 0xffff, y1 = r.y >> 16;
  uint64_t dbits = (uint64_t)__float_as_uint(a.geom.rgbd[g].w) << 32;
  uint32_t j = off;
  for (int ty = y0; ty < y1; ++ty) {
    for (int tx = x0; tx < x1; ++tx, ++j) {
      int tile = ty * a.grid_x + tx;
      uint32_t pos = a.tile_range[tile] + atomicAdd(&a.tile_cursor[tile], 1u);
      a.bin.keys[pos] = dbits | j;
      a.bin.inst_gid[j] = (uint32_t)g;
    }
  }
}

__device__ __forceinline__ void bitonic_sort_smem(uint64_t* s, int n2) {
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        int ixj = i ^ j;
        if (ixj > i) {
          uint64_t x = s[i], y = s[ixj];
          bool asc = (i & k) == 0;
          if ((x > y) == asc) {
            s[i] = y;
            s[ixj] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ int next_pow2(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

// Merge-path split: number of elements taken from A among the first d outputs.
__device__ __forceinline__ int merge_split(const uint64_t* A, int la, const uint64_t* B, int lb, int d) {
  int lo = max(0, d - lb), hi = min(d, la);
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (A[mid] < B[d - mid - 1]) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

struct SortArgs {
  const uint32_t* tile_range;
  BinningView bin;
  int64_t cap;
  const CfgsCounts* counts;
};

// One block per tile. Segments of at most kSortCap instances: bitonic sort in shared
// memory. Larger segments: bitonic-sort kSortCap chunks, then merge them pairwise
// (merge path, ping-pong between keys and keys_alt) inside the block.
__global__ void __launch_bounds__(kSortThreads) k_tile_sort(SortArgs a) {
  __shared__ uint64_t s[kSortCap];
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const uint32_t lo = a.tile_range[blockIdx.x];
  const int n = (int)(a.tile_range[blockIdx.x + 1] - lo);
  if (n == 0) return;
  uint64_t* keys = a.bin.keys + lo;
  if (n <= kSortCap) {
    int n2 = next_pow2(n);
    for (int i = threadIdx.x; i < n2; i += blockDim.x) s[i] = i < n ? keys[i] : ~0ull;
    __syncthreads();
    bitonic_sort_smem(s, n2);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      uint32_t pidx = (uint32_t)s[i];
      a.bin.sorted_pidx[lo + i] = pidx;
      a.bin.sorted_gid[lo + i] = a.bin.inst_gid[pidx];
    }
    return;
  }
  for (int c0 = 0; c0 < n; c0 += kSortCap) {
    int m = min(kSortCap, n - c0);
    int m2 = next_pow2(m);
    for (int i = threadIdx.x; i < m2; i += blockDim.x) s[i] = i < m ? keys[c0 + i] : ~0ull;
    __syncthreads();
    bitonic_sort_smem(s, m2);
    for (int i = threadIdx.x; i < m; i += blockDim.x) keys[c0 + i] = s[i];
    __syncthreads();
  }
  uint64_t* src = keys;
  uint64_t* dst = a.bin.keys_alt + lo;
  for (int width = kSortCap; width < n; width <<= 1) {
    for (int base = 0; base < n; base += 2 * width) {
      int la = min(width, n - base);
      int lb = max(0, min(width, n - base - la));
      const uint64_t* A = src + base;
      const uint64_t* B = A + la;
      uint64_t* out = dst + base;
      int total = la + lb;
      int per = (total + blockDim.x - 1) / blockDim.x;
      int d0 = min(total, (int)threadIdx.x * per);
      int d1 = min(total, d0 + per);
      if (d0 < d1) {
        int i = merge_split(A, la, B, lb, d0);
        int j = d0 - i;
        for (int d = d0; d < d1; ++d) {
          if (j >= lb || (i < la && A[i] < B[j])) out[d] = A[i++];
          else out[d] = B[j++];
        }
      }
    }
    __syncthreads();
    uint64_t* tmp = src;
    src = dst;
    dst = tmp;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    uint32_t pidx = (uint32_t)src[i];
    a.bin.sorted_pidx[lo + i] = pidx;
    a.bin.sorted_gid[lo + i] = a.bin.inst_gid[pidx];
  }
}

struct RenderArgs {
  int W, H, grid_x;
  const float* bg;
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
};

// One block per 16x16 tile, one thread per pixel. Batches of 256 instances are
// gathered into shared memory (per-Gaussian data stays L2-resident); compositing runs
// front to back with the published thresholds; the block leaves as soon as every
// pixel is saturated (block-wide vote).
__global__ void __launch_bounds__(kTilePixels) k_render_fwd(RenderArgs a) {
  __shared__ float2 s_xy[kRenderBatch];
  __shared__ float4 s_co[kRenderBatch];
  __shared__ float4 s_rgbd[kRenderBatch];
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const int tile = blockIdx.x;
  const int px = (tile % a.grid_x) * kTileX + (threadIdx.x % kTileX);
  const int py = (tile / a.grid_x) * kTileY + (threadIdx.x / kTileX);
  const bool inside = px < a.W && py < a.H;
  const float pxf = (float)px, pyf = (float)py;
  const uint32_t lo = a.tile_range[tile];
  const int n = (int)(a.tile_range[tile + 1] - lo);
  bool done = !inside;
  float T = 1.0f, C0 = 0.0f, C1 = 0.0f, C2 = 0.0f, D = 0.0f;
  uint32_t contributor = 0, last = 0;
  for (int base = 0; base < n; base += kRenderBatch) {
    if (__syncthreads_count(done) == kRenderBatch) break;
    int i = base + threadIdx.x;
    if (i < n) {
      uint32_t g = a.sorted_gid[lo + i];
      s_xy[threadIdx.x] = a.xy[g];
      float4 co = a.conic_op[g];
      s_co[threadIdx.x] = make_float4(-0.5f * co.x, -co.y, -0.5f * co.z, co.w);
      s_rgbd[threadIdx.x] = a.rgbd[g];
    }
    __syncthreads();
    const int cnt = min(kRenderBatch, n - base);
    for (int j = 0; !done && j < cnt; ++j) {
      ++contributor;
      float2 m = s_xy[j];
      float4 co = s_co[j];
      float power = gauss_power(co.x, co.y, co.z, m.x - pxf, m.y - pyf);
      if (power > 0.0f) continue;
      float alpha = fminf(CFGS_ALPHA_MAX, co.w * exp_ref(power));
      if (alpha < CFGS_ALPHA_MIN) continue;
      float test_T = T * (1.0f - alpha);
      if (test_T < CFGS_T_MIN) {
        done = true;
        continue;
      }
      float4 c = s_rgbd[j];
      float w = alpha * T;
      C0 = fmaf(c.x, w, C0);
      C1 = fmaf(c.y, w, C1);
      C2 = fmaf(c.z, w, C2);
      D = fmaf(c.w, w, D);
      T = test_T;
      last = contributor;
    }
  }
  if (inside) {
    const size_t HW = (size_t)a.W * a.H;
    const size_t pix = (size_t)py * a.W + px;
    a.final_T[pix] = T;
    a.n_contrib[pix] = last;
    a.out_color[pix] = fmaf(T, __ldg(a.bg + 0), C0);
    a.out_color[HW + pix] = fmaf(T, __ldg(a.bg + 1), C1);
    a.out_color[2 * HW + pix] = fmaf(T, __ldg(a.bg + 2), C2);
    if (a.out_depth) a.out_depth[pix] = D;
    if (a.out_alpha) a.out_alpha[pix] = 1.0f - T;
  }
}

}  // namespace cfgs

using namespace cfgs;

extern "C" int cfgs_bin_forward(const CfgsSettings* s, const CfgsGaussians* g, void* geom, void* image, void* binning,
                                int64_t capacity, void* stream) {
  if (!s || !g || !geom || !image || !binning || capacity < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (s->image_width <= 0 || s->image_height <= 0 || g->num_gaussians < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity > 0x7fffffffll) return CFGS_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  ImageLayout IL(s->image_width, s->image_height);
  ImageView iv(image, s->image_width, s->image_height);
  GeomView gv(geom, g->num_gaussians);
  GeomLayout GL(g->num_gaussians);
  BinningView bv(binning, capacity);
  if (g->num_gaussians > 0) {
    ScatterArgs sa{g->num_gaussians, gv, iv.tile_range, iv.tile_cursor, IL.grid_x, bv, capacity, iv.counts};
    k_scatter<<<GL.num_blocks, kPreprocessBlock, 0, st>>>(sa);
    CFGS_CHECK_LAUNCH(s->debug, st);
  }
  SortArgs so{iv.tile_range, bv, capacity, iv.counts};
  k_tile_sort<<<IL.num_tiles, kSortThreads, 0, st>>>(so);
  CFGS_CHECK_LAUNCH(s->debug, st);
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
  RenderArgs ra;
  ra.W = s->image_width;
  ra.H = s->image_height;
  ra.grid_x = IL.grid_x;
  ra.bg = s->bg;
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
  k_render_fwd<<<IL.num_tiles, kTilePixels, 0, st>>>(ra);
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
