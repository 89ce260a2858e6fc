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
constexpr int kRenderThreads = 128;  // 2 pixels per thread, 4 warps per 16x16 tile
constexpr int kRenderBatch = 128;

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
// 8 bits per pass, in shared memory. Warp w owns the contiguous eighth
// [w n/8, (w+1) n/8) of the segment and walks it 32 elements per round (conflict-free,
// consecutive lanes on consecutive elements). Counting: per round, lanes with equal
// digits find each other with __match_any_sync and the lowest adds their number to the
// warp's column of a [256][8] histogram. A block-wide exclusive scan of the histogram
// in (digit, warp) order gives each warp its first slot per digit. Scatter: per round the
// same match gives each lane its rank among equal digits, the lowest lane advances the
// warp's running slot. Everything before an element in the segment (earlier rounds,
// earlier warps, lower lanes) lands before it: stable. Passes whose digit is the same
// for all elements are skipped. Equal depths then appear in input order, which the
// scatter left arbitrary, so each run of equal depths is re-sorted by pre-sort index:
// the final order is (depth, pre-sort index), unique.
struct RadixSmem {
  uint32_t key[2][kSortCap];
  uint16_t idx[2][kSortCap];
  uint16_t hist[256][kSortThreads / 32];   // counts, then first slots
  uint32_t warp_tot[kSortThreads / 32];
};

__device__ void radix_sort_segment(RadixSmem& S, const uint64_t* keys, int n, int& out_buf) {
  constexpr int kW = kSortThreads / 32;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int per = (n + kW - 1) / kW;
  const int w0 = min(n, warp * per), w1 = min(n, w0 + per);
  for (int i = t; i < n; i += kSortThreads) {
    S.key[0][i] = (uint32_t)(keys[i] >> 32);
    S.idx[0][i] = (uint16_t)i;
  }
  int cur = 0;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int shift = 0; shift < 32; shift += 8) {
    for (int d = t; d < 256 * kW; d += kSortThreads) (&S.hist[0][0])[d] = 0;
    __syncthreads();
    for (int base = w0; base < w1; base += 32) {
      const int i = base + lane;
      const bool act = i < w1;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (act) {
        const uint32_t d = (S.key[cur][i] >> shift) & 255u;
        const unsigned peers = __match_any_sync(am, d);
        if ((peers & lt_mask) == 0) S.hist[d][warp] += (uint16_t)__popc(peers);
      }
    }
    __syncthreads();
    // exclusive scan in (digit, warp) order: thread t owns digit t's 8 warp entries
    uint32_t loc[kW];
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kW; ++w) {
      loc[w] = run;
      run += S.hist[t][w];
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
    const bool trivial_local = run == (uint32_t)n;  // digit t holds every element
    const bool trivial = __syncthreads_or(trivial_local);
    if (trivial) continue;
#pragma unroll
    for (int w = 0; w < kW; ++w) S.hist[t][w] = (uint16_t)(pre + loc[w]);
    __syncthreads();
    const int nxt = cur ^ 1;
    for (int base = w0; base < w1; base += 32) {
      const int i = base + lane;
      const bool act = i < w1;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (act) {
        const uint32_t k = S.key[cur][i];
        const uint32_t d = (k >> shift) & 255u;
        const unsigned peers = __match_any_sync(am, d);
        const int leader = __ffs(peers) - 1;
        const uint32_t slot0 = S.hist[d][warp];
        const uint32_t pos = slot0 + __popc(peers & lt_mask);
        S.key[nxt][pos] = k;
        S.idx[nxt][pos] = S.idx[cur][i];
        __syncwarp(am);
        if (lane == leader) S.hist[d][warp] = (uint16_t)(slot0 + __popc(peers));
        __syncwarp(am);
      }
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

// Front-to-back state of one pixel and one compositing step (the published loop body,
// with the exponential skipped below the alpha threshold — exact, see alpha_threshold).
struct PixelFwd {
  float T, C0, C1, C2, D;
  uint32_t last;
  bool done;
};

__device__ __forceinline__ void composite_step(PixelFwd& p, float pxf, float pyf, const float4& xyt, const float4& co,
                                               const float4* s_rgbd, int j, uint32_t pos1) {
  if (p.done) return;
  const float power = gauss_power(co.x, co.y, co.z, xyt.x - pxf, xyt.y - pyf);
  if (power > 0.0f || power < xyt.z) return;
  const float alpha = fminf(CFGS_ALPHA_MAX, co.w * exp_ref_inrange(power));
  if (alpha < CFGS_ALPHA_MIN) return;
  const float test_T = p.T * (1.0f - alpha);
  if (test_T < CFGS_T_MIN) {
    p.done = true;
    return;
  }
  const float4 c = s_rgbd[j];
  const float w = alpha * p.T;
  p.C0 = fmaf(c.x, w, p.C0);
  p.C1 = fmaf(c.y, w, p.C1);
  p.C2 = fmaf(c.z, w, p.C2);
  p.D = fmaf(c.w, w, p.D);
  p.T = test_T;
  p.last = pos1;
}

// One block of 128 threads per 16x16 tile; warp w covers the 8x8 pixel box
// (8 (w & 1), 8 (w >> 1)) and each lane two pixels of it, rows r and r + 4. Batches of
// 128 instances are gathered into shared memory (per-Gaussian data stays L2-resident).
// Two exact shortcuts skip work whose outcome is known: each warp keeps only the
// instances whose alpha >= 1/255 ellipse can reach its box (box_may_contribute, one test
// per instance and warp), and a pixel skips the exponential when the exponent lies
// below the instance's alpha_threshold. Neither changes a decision of the published
// algorithm, so every output — contributor counts included, which count positions in
// the tile's list — is what the plain per-pixel loop gives. Compositing runs front to
// back; a warp stops when its pixels are saturated and the block when all are.
template <class Scenes>
__global__ void __launch_bounds__(kRenderThreads) k_render_fwd(RenderArgs<Scenes> a) {
  __shared__ float4 s_xyt[kRenderBatch];   // (x, y, alpha threshold, -)
  __shared__ float4 s_co[kRenderBatch];    // (ca, cb, cc, opacity)
  __shared__ float4 s_rgbd[kRenderBatch];
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const int tile = blockIdx.x;
  const SceneDesc& sd = a.scenes.for_tile(tile);
  const int lt = tile - sd.tile_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bx0 = (lt % sd.grid_x) * kTileX + (warp & 1) * 8;
  const int by0 = (lt / sd.grid_x) * kTileY + (warp >> 1) * 8;
  const int px = bx0 + (lane & 7), py0 = by0 + (lane >> 3), py1 = py0 + 4;
  const float bxf0 = (float)bx0, bxf1 = (float)(bx0 + 7), byf0 = (float)by0, byf1 = (float)(by0 + 7);
  const bool in0 = px < sd.W && py0 < sd.H, in1 = px < sd.W && py1 < sd.H;
  const float pxf = (float)px, pyf0 = (float)py0, pyf1 = (float)py1;
  const uint32_t lo = a.tile_range[tile];
  const int n = (int)(a.tile_range[tile + 1] - lo);
  PixelFwd p0{1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0u, !in0};
  PixelFwd p1{1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0u, !in1};
  for (int base = 0; base < n; base += kRenderBatch) {
    if (__syncthreads_count(p0.done && p1.done) == kRenderThreads) break;
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
      if (__all_sync(0xffffffffu, p0.done && p1.done)) break;
      uint32_t mk = keep[r];
      while (mk) {
        const int j = r * 32 + __ffs(mk) - 1;
        mk &= mk - 1;
        const float4 xyt = s_xyt[j];
        const float4 co = s_co[j];
        const uint32_t pos1 = (uint32_t)(base + j + 1);
        composite_step(p0, pxf, pyf0, xyt, co, s_rgbd, j, pos1);
        composite_step(p1, pxf, pyf1, xyt, co, s_rgbd, j, pos1);
      }
    }
  }
  const size_t HW = (size_t)sd.W * sd.H;
  float* col = a.out_color + 3 * (size_t)sd.pix_base;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const PixelFwd& p = q ? p1 : p0;
    const int py = q ? py1 : py0;
    if (!(q ? in1 : in0)) continue;
    const size_t pix = (size_t)py * sd.W + px;
    const size_t gp = (size_t)sd.pix_base + pix;
    a.final_T[gp] = p.T;
    a.n_contrib[gp] = p.last;
    col[pix] = fmaf(p.T, __ldg(sd.bg + 0), p.C0);
    col[HW + pix] = fmaf(p.T, __ldg(sd.bg + 1), p.C1);
    col[2 * HW + pix] = fmaf(p.T, __ldg(sd.bg + 2), p.C2);
    if (a.out_depth) a.out_depth[gp] = p.D;
    if (a.out_alpha) a.out_alpha[gp] = 1.0f - p.T;
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
  k_render_fwd<Scenes><<<tiles, kRenderThreads, 0, st>>>(a);
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
