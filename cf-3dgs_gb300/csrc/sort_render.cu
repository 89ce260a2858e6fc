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
// Every kernel is a template over the scene accessor (one scene for the drop-in path,
// a descriptor table for batched solves); the arithmetic is the same for both.
// Compiled with -fmad=false; the fmaf() calls are the only fused operations, and the
// CPU oracle performs the same sequence.
#include "cfgs_internal.cuh"
#include "kernels.cuh"

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

// One thread per Gaussian slot (the preprocess's 256-wide partition, so the block
// prefixes line up) assigns pre-sort instance indices in Gaussian order, row-major over
// the tile rectangle. The instances are then emitted warp-cooperatively: the warp's
// instances are dealt out 32 per round, one per lane, so every round issues 32
// independent slot reservations; lanes that hit the same tile in a round share one
// atomicAdd (match_any). Positions inside a tile's range are arbitrary here — the tile
// sort imposes the order.
template <class Scenes>
__global__ void __launch_bounds__(kPreprocessBlock) k_scatter(ScatterArgs<Scenes> a) {
  __shared__ uint32_t sh[kPreprocessBlock / 32];
  __shared__ uint32_t s_start[kPreprocessBlock];
  __shared__ uint32_t s_off[kPreprocessBlock];
  __shared__ uint2 s_rect[kPreprocessBlock];
  __shared__ uint32_t s_dbits[kPreprocessBlock];
  if ((int64_t)a.counts->num_rendered > a.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.counts->flags, CFGS_FLAG_CAPACITY_OVERFLOW);
    return;
  }
  const SceneDesc& sd = a.scenes.for_block(blockIdx.x);
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, wbase = threadIdx.x & ~31;
  uint32_t t = g < a.total_slots ? a.geom.touched[g] : 0u;
  uint32_t tot;
  uint32_t off = a.geom.block_prefix[blockIdx.x] + block_excl_scan_256(t, sh, &tot);
  if (g < a.total_slots) a.geom.offset[g] = off;
  // warp-inclusive scan of t -> each lane's first warp-local instance
  uint32_t x = t;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const uint32_t warp_total = __shfl_sync(0xffffffffu, x, 31);
  s_start[threadIdx.x] = x - t;
  s_off[threadIdx.x] = off;
  s_rect[threadIdx.x] = t ? a.geom.rect[g] : make_uint2(0u, 0u);
  s_dbits[threadIdx.x] = t ? __float_as_uint(a.geom.rgbd[g].w) : 0u;
  __syncwarp();
  uint32_t* cursor = a.tile_cursor;
  const uint32_t* range = a.tile_range;
  for (uint32_t base = 0; base < warp_total; base += 32) {
    const uint32_t w = base + lane;
    const bool active = w < warp_total;
    uint32_t tile = 0xffffffffu, pidx = 0, gid = 0, dbits = 0;
    if (active) {
      // owner lane: the last lane whose start <= w (lanes with t == 0 share starts)
      int lo = 0, hi = 31;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (s_start[wbase + mid] <= w) lo = mid;
        else hi = mid - 1;
      }
      const int ol = wbase + lo;
      const uint32_t j = w - s_start[ol];
      const uint2 r = s_rect[ol];
      const uint32_t x0 = r.x & 0xffffu, y0 = r.x >> 16, x1 = r.y & 0xffffu;
      const uint32_t rw = x1 - x0;
      const uint32_t ty = y0 + j / rw, tx = x0 + j % rw;
      tile = (uint32_t)sd.tile_base + ty * (uint32_t)sd.grid_x + tx;
      pidx = s_off[ol] + j;
      gid = (uint32_t)((int64_t)blockIdx.x * blockDim.x + ol);
      dbits = s_dbits[ol];
    }
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (active) {
      const unsigned peers = __match_any_sync(act, tile);
      const int leader = __ffs(peers) - 1;
      const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
      uint32_t slot = 0;
      if (lane == leader) slot = atomicAdd(&cursor[tile], (uint32_t)__popc(peers));
      slot = __shfl_sync(peers, slot, leader) + rank;
      const uint32_t pos = range[tile] + slot;
      a.bin.keys[pos] = ((uint64_t)dbits << 32) | pidx;
      a.bin.inst_gid[pidx] = gid;
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

// Stable LSD radix sort of a tile segment (n <= kSortCap) by the 32-bit depth bits,
// 4 bits per pass, in shared memory: each thread owns a run of consecutive elements,
// counts its digits into its own column of a [16][256] table, a block-wide exclusive
// scan of the table in digit-major order gives every (digit, thread) its first output
// slot, and the thread writes its elements in order (stable). Passes whose digit is the
// same for all elements are skipped. Equal depths then appear in input order, which the
// scatter left arbitrary, so each run of equal depths is re-sorted by pre-sort index:
// the final order is (depth, pre-sort index), unique.
struct RadixSmem {
  uint32_t key[2][kSortCap];
  uint16_t idx[2][kSortCap];
  uint32_t cnt[16][kSortThreads + 1];
  uint32_t warp_tot[kSortThreads / 32];
  int trivial;
};

__device__ void radix_sort_segment(RadixSmem& S, const uint64_t* keys, int n, int& out_buf) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int E = (n + kSortThreads - 1) / kSortThreads;
  const int b0 = min(n, t * E), b1 = min(n, b0 + E);
  for (int i = t; i < n; i += kSortThreads) {
    S.key[0][i] = (uint32_t)(keys[i] >> 32);
    S.idx[0][i] = (uint16_t)i;
  }
  int cur = 0;
  for (int shift = 0; shift < 32; shift += 4) {
#pragma unroll
    for (int d = 0; d < 16; ++d) S.cnt[d][t] = 0;
    __syncthreads();
    for (int i = b0; i < b1; ++i) S.cnt[(S.key[cur][i] >> shift) & 15u][t]++;
    __syncthreads();
    // exclusive scan of cnt in digit-major order; thread t owns flat entries [16t, 16t+16)
    uint32_t loc[16];
    uint32_t run = 0;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int f = 16 * t + u;
      loc[u] = run;
      run += S.cnt[f >> 8][f & 255];
    }
    uint32_t x = run;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) S.warp_tot[warp] = x;
    __syncthreads();
    uint32_t pre = x - run;
    for (int w = 0; w < warp; ++w) pre += S.warp_tot[w];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int f = 16 * t + u;
      S.cnt[f >> 8][f & 255] = pre + loc[u];
    }
    __syncthreads();
    bool trivial = false;  // one digit holds every element: the pass changes nothing
#pragma unroll
    for (int d = 0; d < 16; ++d) {
      const uint32_t start = S.cnt[d][0], end = d < 15 ? S.cnt[d + 1][0] : (uint32_t)n;
      trivial |= (end - start == (uint32_t)n);
    }
    if (trivial) {  // uniform: every thread read the same bucket starts
      __syncthreads();
      continue;
    }
    const int nxt = cur ^ 1;
    for (int i = b0; i < b1; ++i) {
      const uint32_t k = S.key[cur][i];
      const uint32_t pos = S.cnt[(k >> shift) & 15u][t]++;
      S.key[nxt][pos] = k;
      S.idx[nxt][pos] = S.idx[cur][i];
    }
    __syncthreads();
    cur = nxt;
  }
  // runs of equal depth: insertion sort by pre-sort index (the key's low 32 bits)
  for (int i = t; i < n; i += kSortThreads) {
    const uint32_t k = S.key[cur][i];
    const bool start = (i == 0 || S.key[cur][i - 1] != k) && (i + 1 < n && S.key[cur][i + 1] == k);
    if (!start) continue;
    int e = i + 1;
    while (e < n && S.key[cur][e] == k) ++e;
    for (int p = i + 1; p < e; ++p) {
      const uint16_t v = S.idx[cur][p];
      const uint32_t pv = (uint32_t)keys[v];
      int q = p - 1;
      while (q >= i && (uint32_t)keys[S.idx[cur][q]] > pv) {
        S.idx[cur][q + 1] = S.idx[cur][q];
        --q;
      }
      S.idx[cur][q + 1] = v;
    }
  }
  __syncthreads();
  out_buf = cur;
}

// One block per tile (global tile index: scene-agnostic). Segments of at most kSortCap
// instances: radix sort in shared memory (above). Larger segments: bitonic-sort
// kSortCap chunks, then merge them pairwise (merge path, ping-pong between keys and
// keys_alt) inside the block.
__global__ void __launch_bounds__(kSortThreads) k_tile_sort(SortArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* s = reinterpret_cast<uint64_t*>(smem_raw);
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const uint32_t lo = a.tile_range[blockIdx.x];
  const int n = (int)(a.tile_range[blockIdx.x + 1] - lo);
  if (n == 0) return;
  uint64_t* keys = a.bin.keys + lo;
  if (n <= kSortCap) {
    RadixSmem& S = *reinterpret_cast<RadixSmem*>(smem_raw);
    int buf = 0;
    radix_sort_segment(S, keys, n, buf);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      uint32_t pidx = (uint32_t)keys[S.idx[buf][i]];
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

// One block per 16x16 tile, one thread per pixel; warp w covers the 8x4 pixel box
// (8 (w & 1), 4 (w >> 1)) of the tile. Batches of 256 instances are gathered into shared
// memory (per-Gaussian data stays L2-resident). Two exact shortcuts skip work whose
// outcome is known: each warp keeps only the instances whose alpha >= 1/255 ellipse can
// reach its box (box_may_contribute, one test per instance and warp), and a pixel skips
// the exponential when the exponent lies below the instance's alpha_threshold. Neither
// changes a decision of the published algorithm, so every output — contributor counts
// included, which count positions in the tile's list — is what the plain loop gives.
// Compositing runs front to back; a warp stops when its pixels are saturated and the
// block when all are.
template <class Scenes>
__global__ void __launch_bounds__(kTilePixels) k_render_fwd(RenderArgs<Scenes> a) {
  __shared__ float4 s_xyt[kRenderBatch];   // (x, y, alpha threshold, -)
  __shared__ float4 s_co[kRenderBatch];    // (ca, cb, cc, opacity)
  __shared__ float4 s_rgbd[kRenderBatch];
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const int tile = blockIdx.x;
  const SceneDesc& sd = a.scenes.for_tile(tile);
  const int lt = tile - sd.tile_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bx0 = (lt % sd.grid_x) * kTileX + (warp & 1) * 8;
  const int by0 = (lt / sd.grid_x) * kTileY + (warp >> 1) * 4;
  const int px = bx0 + (lane & 7), py = by0 + (lane >> 3);
  const float bxf0 = (float)bx0, bxf1 = (float)(bx0 + 7), byf0 = (float)by0, byf1 = (float)(by0 + 3);
  const bool inside = px < sd.W && py < sd.H;
  const float pxf = (float)px, pyf = (float)py;
  const uint32_t lo = a.tile_range[tile];
  const int n = (int)(a.tile_range[tile + 1] - lo);
  bool done = !inside;
  float T = 1.0f, C0 = 0.0f, C1 = 0.0f, C2 = 0.0f, D = 0.0f;
  uint32_t last = 0;
  for (int base = 0; base < n; base += kRenderBatch) {
    if (__syncthreads_count(done) == kRenderBatch) break;
    int i = base + threadIdx.x;
    if (i < n) {
      uint32_t g = a.sorted_gid[lo + i];
      float2 m = a.xy[g];
      float4 co = a.conic_op[g];
      s_xyt[threadIdx.x] = make_float4(m.x, m.y, alpha_threshold(co.w), 0.0f);
      s_co[threadIdx.x] = make_float4(-0.5f * co.x, -co.y, -0.5f * co.z, co.w);
      s_rgbd[threadIdx.x] = a.rgbd[g];
    }
    __syncthreads();
    const int cnt = min(kRenderBatch, n - base);
    uint32_t keep[kRenderBatch / 32];
#pragma unroll
    for (int r = 0; r < kRenderBatch / 32; ++r) {
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
    for (int r = 0; r < kRenderBatch / 32; ++r) {
      if (__all_sync(0xffffffffu, done)) break;
      uint32_t mk = keep[r];
      while (mk) {
        const int j = r * 32 + __ffs(mk) - 1;
        mk &= mk - 1;
        if (done) continue;
        const float4 xyt = s_xyt[j];
        const float4 co = s_co[j];
        const float power = gauss_power(co.x, co.y, co.z, xyt.x - pxf, xyt.y - pyf);
        if (power > 0.0f || power < xyt.z) continue;
        const float alpha = fminf(CFGS_ALPHA_MAX, co.w * exp_ref_inrange(power));
        if (alpha < CFGS_ALPHA_MIN) continue;
        const float test_T = T * (1.0f - alpha);
        if (test_T < CFGS_T_MIN) {
          done = true;
          continue;
        }
        const float4 c = s_rgbd[j];
        const float w = alpha * T;
        C0 = fmaf(c.x, w, C0);
        C1 = fmaf(c.y, w, C1);
        C2 = fmaf(c.z, w, C2);
        D = fmaf(c.w, w, D);
        T = test_T;
        last = (uint32_t)(base + j + 1);
      }
    }
  }
  if (inside) {
    const size_t HW = (size_t)sd.W * sd.H;
    const size_t pix = (size_t)py * sd.W + px;
    const size_t gp = (size_t)sd.pix_base + pix;
    a.final_T[gp] = T;
    a.n_contrib[gp] = last;
    float* col = a.out_color + 3 * (size_t)sd.pix_base;
    col[pix] = fmaf(T, __ldg(sd.bg + 0), C0);
    col[HW + pix] = fmaf(T, __ldg(sd.bg + 1), C1);
    col[2 * HW + pix] = fmaf(T, __ldg(sd.bg + 2), C2);
    if (a.out_depth) a.out_depth[gp] = D;
    if (a.out_alpha) a.out_alpha[gp] = 1.0f - T;
  }
}

// ---- launchers (shared by the drop-in entry points and the batched engine) --------
template <class Scenes>
void launch_scatter(const ScatterArgs<Scenes>& a, int blocks, cudaStream_t st) {
  k_scatter<Scenes><<<blocks, kPreprocessBlock, 0, st>>>(a);
}
void launch_tile_sort(const SortArgs& a, int tiles, cudaStream_t st) {
  constexpr size_t kSmem = sizeof(RadixSmem) > sizeof(uint64_t) * kSortCap ? sizeof(RadixSmem)
                                                                          : sizeof(uint64_t) * kSortCap;
  static bool attr_set = false;  // a function attribute: set once per process (before any capture)
  if (!attr_set) {
    cudaFuncSetAttribute(k_tile_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    attr_set = true;
  }
  k_tile_sort<<<tiles, kSortThreads, kSmem, st>>>(a);
}
template <class Scenes>
void launch_render_fwd(const RenderArgs<Scenes>& a, int tiles, cudaStream_t st) {
  k_render_fwd<Scenes><<<tiles, kTilePixels, 0, st>>>(a);
}
template void launch_scatter<SingleScene>(const ScatterArgs<SingleScene>&, int, cudaStream_t);
template void launch_scatter<SceneTable>(const ScatterArgs<SceneTable>&, int, cudaStream_t);
template void launch_render_fwd<SingleScene>(const RenderArgs<SingleScene>&, int, cudaStream_t);
template void launch_render_fwd<SceneTable>(const RenderArgs<SceneTable>&, int, cudaStream_t);

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
    ScatterArgs<SingleScene> sa;
    sa.scenes.d = single_scene_desc(s, g->num_gaussians, g->sh_coeffs);
    sa.total_slots = g->num_gaussians;
    sa.geom = gv;
    sa.tile_range = iv.tile_range;
    sa.tile_cursor = iv.tile_cursor;
    sa.bin = bv;
    sa.cap = capacity;
    sa.counts = iv.counts;
    launch_scatter(sa, GL.num_blocks, st);
    CFGS_CHECK_LAUNCH(s->debug, st);
  }
  SortArgs so{iv.tile_range, bv, capacity, iv.counts};
  launch_tile_sort(so, IL.num_tiles, st);
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
