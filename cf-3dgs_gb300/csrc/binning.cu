// Forward phase 2: binning — the list of (tile, Gaussian) instances in the order the
// compositing reads them: by tile, within a tile by depth, equal depths by Gaussian id.
//
// Upstream emits K 64-bit keys (tile << 32 | depth bits) in Gaussian order and runs
// one global stable radix sort over 32 + log2(tiles) bits. Here the depth part is
// sorted once per Gaussian instead of once per instance:
//   1. depth sort: stable LSD radix sort of the N depth keys (4 passes of 8 bits), so
//      the Gaussians come out by (depth, id);
//   2. emission: the instances are written in that order (a Gaussian's tiles in
//      row-major order of its tile rectangle), with coalesced stores; an instance's
//      index is its position in this list;
//   3. tile sort: stable LSD radix sort of the instances by tile index alone
//      (ceil(log2 tiles) bits, at most 8 per pass: 2 passes at 1080p).
// A stable sort by tile of a list ordered by (depth, id) is ordered by (tile, depth,
// id): exactly the stable sort of upstream's keys over instances emitted by id. The
// last tile pass also counts the instances of every tile (runs of equal tiles), and a
// scan turns the counts into tile ranges.
//
// Every radix pass is three launches over chunks of kSortChunk elements: count (digit
// histogram per chunk), scan (per digit, over chunks: the chunk's first global slot),
// scatter (rank inside the chunk, stage in shared memory by digit, then write each
// digit's run to its global slots). Ranking inside a chunk is stable: warp w owns the
// contiguous slice [w C/8, (w+1) C/8) and walks it 32 elements per round; lanes with
// equal digits find each other with __match_any_sync.
#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = kSortChunk / kSortThreads;  // 16 elements per thread
constexpr int kWarpSlice = kSortChunk / kSortWarps;     // 512 elements per warp

// One radix pass. Keys come from key_in, or (depth mode, key_in == NULL) from the
// geometry: the depth bits of Gaussians that touch a tile, ~0 for the others, so they
// sort last. Payloads come from val_in / aux_in, or are the element's own index when
// those are NULL.
struct SortPass {
  const uint32_t* key_in;
  const uint32_t* val_in;
  const uint32_t* aux_in;
  const float4* depth_rgbd;    // depth mode
  const uint32_t* depth_touched;
  uint32_t* key_out;           // NULL: keys are not written (last pass)
  uint32_t* val_out;
  uint32_t* aux_out;           // NULL: one payload
  uint32_t* tile_count;        // last tile pass: instances per tile
  int shift, bits;
  int64_t n;                   // element count, when counts is NULL
  const CfgsCounts* counts;    // element count = num_rendered (nothing to do above cap)
  int64_t cap;
  int64_t num_chunks;          // chunks covered by the grid
  uint32_t* chunk_counts;      // [1 << bits][num_chunks]
  uint32_t* digit_totals;      // [1 << bits], zero before the count launch
};

__device__ __forceinline__ int64_t pass_elements(const SortPass& p) {
  if (!p.counts) return p.n;
  const int64_t k = (int64_t)p.counts->num_rendered;
  return k > p.cap ? 0 : k;
}

__device__ __forceinline__ uint32_t pass_key(const SortPass& p, int64_t i) {
  if (p.key_in) return p.key_in[i];
  return p.depth_touched[i] ? __float_as_uint(p.depth_rgbd[i].w) : 0xffffffffu;
}

__global__ void __launch_bounds__(kSortThreads) k_sort_count(SortPass p) {
  __shared__ uint32_t hist[kSortWarps][kSortDigits];
  const int64_t n = pass_elements(p);
  const int64_t c0 = (int64_t)blockIdx.x * kSortChunk;
  if (c0 >= n) return;
  const int cnt = (int)min((int64_t)kSortChunk, n - c0);
  const int ndig = 1 << p.bits;
  const uint32_t mask = (uint32_t)ndig - 1u;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kSortWarps * kSortDigits; i += kSortThreads) (&hist[0][0])[i] = 0u;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll 4
  for (int k = 0; k < kSortItems; ++k) {
    const int i = warp * kWarpSlice + k * 32 + lane;
    const bool act = i < cnt;
    const unsigned am = __ballot_sync(0xffffffffu, act);
    if (act) {
      const uint32_t d = (pass_key(p, c0 + i) >> p.shift) & mask;
      const unsigned peers = __match_any_sync(am, d);
      if ((peers & lt) == 0) hist[warp][d] += (uint32_t)__popc(peers);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < ndig; d += kSortThreads) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) s += hist[w][d];
    p.chunk_counts[(size_t)d * p.num_chunks + blockIdx.x] = s;
    if (s) atomicAdd(&p.digit_totals[d], s);
  }
}

// Block-wide inclusive scan of one value per thread (blockDim.x <= 1024); returns the
// inclusive prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t v, uint32_t* sh, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nw ? sh[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh[32 + lane] = w;
  }
  __syncthreads();
  const uint32_t r = x + (warp > 0 ? sh[32 + warp - 1] : 0u);
  *total = sh[32 + nw - 1];
  __syncthreads();
  return r;
}

// One block per digit d: chunk_counts[d][c] becomes the global slot of digit d's first
// element in chunk c = (elements with a smaller digit) + (digit-d elements of earlier
// chunks).
__global__ void __launch_bounds__(1024) k_sort_scan(SortPass p) {
  __shared__ uint32_t sh[64];
  const int64_t n = pass_elements(p);
  if (n <= 0) return;
  const int d = blockIdx.x;
  const int64_t nc = (n + kSortChunk - 1) / kSortChunk;
  uint32_t tot;
  const uint32_t below = (int)threadIdx.x < d ? p.digit_totals[threadIdx.x] : 0u;
  block_inclusive_scan(below, sh, &tot);
  uint32_t carry = tot;
  uint32_t* col = p.chunk_counts + (size_t)d * p.num_chunks;
  for (int64_t c0 = 0; c0 < nc; c0 += blockDim.x) {
    const int64_t c = c0 + threadIdx.x;
    const uint32_t v = c < nc ? col[c] : 0u;
    const uint32_t incl = block_inclusive_scan(v, sh, &tot);
    if (c < nc) col[c] = carry + incl - v;
    carry += tot;
  }
}

// Dynamic shared memory of the scatter: staged keys and payloads, per-warp digit
// counters, per-digit block-local starts and global slots.
inline size_t scatter_smem(bool aux) {
  return sizeof(uint32_t) * ((aux ? 3 : 2) * (size_t)kSortChunk + (size_t)kSortWarps * kSortDigits + 2 * kSortDigits);
}

__global__ void __launch_bounds__(kSortThreads, 2) k_sort_scatter(SortPass p) {
  extern __shared__ __align__(16) uint32_t smem[];
  const bool has_aux = p.aux_out != nullptr;
  uint32_t* s_key = smem;
  uint32_t* s_val = s_key + kSortChunk;
  uint32_t* s_aux = s_val + kSortChunk;
  uint32_t* s_whist = s_val + (has_aux ? 2 : 1) * kSortChunk;  // [warp][digit]
  uint32_t* s_start = s_whist + kSortWarps * kSortDigits;       // block-local first position of a digit
  uint32_t* s_slot = s_start + kSortDigits;                      // global first slot of a digit
  __shared__ uint32_t sh[64];

  const int64_t n = pass_elements(p);
  const int64_t c0 = (int64_t)blockIdx.x * kSortChunk;
  if (c0 >= n) return;
  const int cnt = (int)min((int64_t)kSortChunk, n - c0);
  const int ndig = 1 << p.bits;
  const uint32_t mask = (uint32_t)ndig - 1u;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int i = t; i < kSortWarps * kSortDigits; i += kSortThreads) s_whist[i] = 0u;
  __syncthreads();

  // rank of every element among the equal digits of its warp's slice
  uint32_t key[kSortItems], rank[kSortItems];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const int i = warp * kWarpSlice + k * 32 + lane;
    const bool act = i < cnt;
    const unsigned am = __ballot_sync(0xffffffffu, act);
    key[k] = 0u;
    rank[k] = 0u;
    if (act) {
      key[k] = pass_key(p, c0 + i);
      const uint32_t d = (key[k] >> p.shift) & mask;
      const unsigned peers = __match_any_sync(am, d);
      const uint32_t before = s_whist[warp * kSortDigits + d];
      rank[k] = before + (uint32_t)__popc(peers & lt);
      __syncwarp(am);
      if ((peers & lt) == 0) s_whist[warp * kSortDigits + d] = before + (uint32_t)__popc(peers);
      __syncwarp(am);
    }
  }
  __syncthreads();

  // digit t: warp offsets inside the digit, block-local start, global slot
  uint32_t dsum = 0;
  if (t < ndig) {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = s_whist[w * kSortDigits + t];
      s_whist[w * kSortDigits + t] = dsum;
      dsum += c;
    }
  }
  uint32_t tot;
  const uint32_t incl = block_inclusive_scan(dsum, sh, &tot);
  if (t < ndig) {
    s_start[t] = incl - dsum;
    s_slot[t] = dsum ? p.chunk_counts[(size_t)t * p.num_chunks + blockIdx.x] : 0u;
  }
  __syncthreads();

  // stage in block-local sorted order
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    const int i = warp * kWarpSlice + k * 32 + lane;
    if (i < cnt) {
      const uint32_t d = (key[k] >> p.shift) & mask;
      const uint32_t pos = s_start[d] + s_whist[warp * kSortDigits + d] + rank[k];
      const int64_t gi = c0 + i;
      s_key[pos] = key[k];
      s_val[pos] = p.val_in ? p.val_in[gi] : (uint32_t)gi;
      if (has_aux) s_aux[pos] = p.aux_in ? p.aux_in[gi] : (uint32_t)gi;
    }
  }
  __syncthreads();

  // each digit's run goes to consecutive global slots
  for (int q = t; q < cnt; q += kSortThreads) {
    const uint32_t kk = s_key[q];
    const uint32_t d = (kk >> p.shift) & mask;
    const size_t g = (size_t)s_slot[d] + (uint32_t)q - s_start[d];
    if (p.key_out) p.key_out[g] = kk;
    p.val_out[g] = s_val[q];
    if (has_aux) p.aux_out[g] = s_aux[q];
    if (p.tile_count) {
      // The chunk is fully sorted now (its input was sorted by the lower digits), so
      // equal tiles form runs: a run [b, e) adds e - b.
      if (q == 0 || s_key[q - 1] != kk) atomicSub(&p.tile_count[kk], (uint32_t)q);
      if (q == cnt - 1 || s_key[q + 1] != kk) atomicAdd(&p.tile_count[kk], (uint32_t)(q + 1));
    }
  }
}

// Instances of every 256 depth-ordered Gaussians (the emission's block prefix).
__global__ void __launch_bounds__(kPreprocessBlock) k_rank_sums(const uint32_t* order, const uint32_t* touched,
                                                                int64_t total_slots, uint32_t* rank_sums) {
  __shared__ uint32_t sh[64];
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t v = r < total_slots ? touched[order[r]] : 0u;
  uint32_t tot;
  block_inclusive_scan(v, sh, &tot);
  if (threadIdx.x == 0) rank_sums[blockIdx.x] = tot;
}

// One thread per depth-ordered Gaussian; the block's first instance index is the sum
// of the earlier blocks' rank_sums, the thread's is that plus a block scan. The
// instances are then written warp-cooperatively: the warp's instances are dealt out
// 32 per round, one per lane, so the stores of a round are consecutive.
template <class Scenes>
__global__ void __launch_bounds__(kPreprocessBlock) k_emit(EmitArgs<Scenes> a) {
  __shared__ uint32_t sh[64];
  __shared__ uint32_t s_start[kPreprocessBlock];
  __shared__ uint32_t s_first[kPreprocessBlock];
  __shared__ uint32_t s_gid[kPreprocessBlock];
  __shared__ uint2 s_rect[kPreprocessBlock];
  __shared__ uint2 s_scene[kPreprocessBlock];  // (tile_base, grid_x)
  if ((int64_t)a.counts->num_rendered > a.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.counts->flags, CFGS_FLAG_CAPACITY_OVERFLOW);
    return;
  }
  uint32_t pre = 0, tot;
  for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) pre += a.rank_sums[b];
  block_inclusive_scan(pre, sh, &tot);
  const uint32_t block_first = tot;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, wbase = threadIdx.x & ~31;
  uint32_t g = 0, nt = 0;
  if (r < a.total_slots) {
    g = a.order[r];
    nt = a.geom.touched[g];
  }
  const uint32_t first = block_first + block_inclusive_scan(nt, sh, &tot) - nt;
  if (nt) {
    a.geom.offset[g] = first;
    const SceneDesc& sd = a.scenes.for_gaussian(g);
    s_rect[threadIdx.x] = a.geom.rect[g];
    s_scene[threadIdx.x] = make_uint2((uint32_t)sd.tile_base, (uint32_t)sd.grid_x);
  }
  // warp-inclusive scan of nt -> each lane's first warp-local instance
  uint32_t x = nt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const uint32_t warp_total = __shfl_sync(0xffffffffu, x, 31);
  s_start[threadIdx.x] = x - nt;
  s_first[threadIdx.x] = first;
  s_gid[threadIdx.x] = g;
  __syncwarp();
  for (uint32_t base = 0; base < warp_total; base += 32) {
    const uint32_t w = base + lane;
    if (w >= warp_total) break;
    // owner lane: the last lane whose start <= w (lanes with nt == 0 share starts)
    int lo = 0, hi = 31;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_start[wbase + mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    const int ol = wbase + lo;
    const uint32_t j = w - s_start[ol];
    const uint2 rc = s_rect[ol];
    const uint32_t x0 = rc.x & 0xffffu, y0 = rc.x >> 16, x1 = rc.y & 0xffffu;
    const uint32_t rw = x1 - x0;
    const uint32_t ty = y0 + j / rw, tx = x0 + j % rw;
    const uint2 sc = s_scene[ol];
    const uint32_t q = s_first[ol] + j;
    a.bin.key[0][q] = sc.x + ty * sc.y + tx;
    a.bin.gid[0][q] = s_gid[ol];
  }
}

// Tile ranges from the per-tile instance counts (one block).
__global__ void __launch_bounds__(1024) k_tile_ranges(const uint32_t* tile_count, uint32_t* tile_range, int num_tiles) {
  __shared__ uint32_t sh[64];
  uint32_t carry = 0, tot;
  for (int base = 0; base < num_tiles; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < num_tiles ? tile_count[i] : 0u;
    const uint32_t incl = block_inclusive_scan(v, sh, &tot);
    if (i < num_tiles) tile_range[i] = carry + incl - v;
    carry += tot;
  }
  if (threadIdx.x == 0) tile_range[num_tiles] = carry;
}

namespace {

bool g_scatter_attr_set = false;

int launch_pass(const SortPass& p, cudaStream_t st) {
  if (!g_scatter_attr_set) {
    if (cudaFuncSetAttribute(k_sort_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scatter_smem(true)) !=
        cudaSuccess)
      return CFGS_ERR_LAUNCH;
    g_scatter_attr_set = true;
  }
  const int grid = (int)p.num_chunks;
  k_sort_count<<<grid, kSortThreads, 0, st>>>(p);
  k_sort_scan<<<1 << p.bits, 1024, 0, st>>>(p);
  k_sort_scatter<<<grid, kSortThreads, scatter_smem(p.aux_out != nullptr), st>>>(p);
  return CFGS_OK;
}

}  // namespace

// Tile-key digits: the fewest passes of at most 8 bits that cover the tile index, split
// evenly.
void tile_sort_plan(int64_t num_tiles, int* passes, int* width) {
  int bits = 1;
  while (bits < 31 && ((int64_t)1 << bits) < num_tiles) ++bits;
  *passes = (bits + 7) / 8;
  *width = (bits + *passes - 1) / *passes;
}

template <class Scenes>
int launch_binning(const BinArgs<Scenes>& a, cudaStream_t st) {
  const GeomView& gv = a.geom;
  const BinningView& bv = a.bin;
  if (cudaMemsetAsync(gv.depth_totals, 0, sizeof(uint32_t) * kSortDigits * kDepthPasses, st) != cudaSuccess ||
      cudaMemsetAsync(bv.totals, 0, sizeof(uint32_t) * kSortDigits * kMaxTilePasses, st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  const int64_t slots = a.total_slots;
  if (slots > 0) {
    // 1. depth sort of the Gaussians: geometry -> 0 -> 1 -> 0 -> depth_val[1]
    int src = -1;
    for (int pass = 0; pass < kDepthPasses; ++pass) {
      SortPass p{};
      const bool last = pass == kDepthPasses - 1;
      const int dst = src == 0 ? 1 : 0;
      p.key_in = src < 0 ? nullptr : gv.depth_key[src];
      p.val_in = src < 0 ? nullptr : gv.depth_val[src];
      p.depth_rgbd = gv.rgbd;
      p.depth_touched = gv.touched;
      p.key_out = last ? nullptr : gv.depth_key[dst];
      p.val_out = last ? gv.depth_val[1] : gv.depth_val[dst];
      p.shift = 8 * pass;
      p.bits = 8;
      p.n = slots;
      p.cap = slots;
      p.num_chunks = sort_chunks(slots);
      p.chunk_counts = gv.depth_counts;
      p.digit_totals = gv.depth_totals + kSortDigits * pass;
      int s = launch_pass(p, st);
      if (s != CFGS_OK) return s;
      src = dst;
    }
    // 2. emission in depth order
    const int rank_blocks = (int)((slots + kPreprocessBlock - 1) / kPreprocessBlock);
    k_rank_sums<<<rank_blocks, kPreprocessBlock, 0, st>>>(gv.depth_val[1], gv.touched, slots, gv.rank_sums);
    EmitArgs<Scenes> e;
    e.scenes = a.scenes;
    e.total_slots = slots;
    e.order = gv.depth_val[1];
    e.rank_sums = gv.rank_sums;
    e.geom = gv;
    e.bin = bv;
    e.cap = a.cap;
    e.counts = a.counts;
    k_emit<Scenes><<<rank_blocks, kPreprocessBlock, 0, st>>>(e);
  }
  // 3. tile sort of the instances: 0 -> 1 -> 0 ... -> sorted
  int passes, width;
  tile_sort_plan(a.num_tiles, &passes, &width);
  const int total_bits = passes * width;
  (void)total_bits;
  int src = 0;
  for (int pass = 0; pass < passes; ++pass) {
    SortPass p{};
    const bool last = pass == passes - 1;
    const int dst = src ^ 1;
    p.key_in = bv.key[src];
    p.val_in = bv.gid[src];
    p.aux_in = pass == 0 ? nullptr : bv.pidx[src];
    p.key_out = last ? nullptr : bv.key[dst];
    p.val_out = last ? bv.sorted_gid : bv.gid[dst];
    p.aux_out = last ? bv.sorted_pidx : bv.pidx[dst];
    p.tile_count = last ? a.tile_count : nullptr;
    p.shift = width * pass;
    p.bits = width;
    p.counts = a.counts;
    p.cap = a.cap;
    p.num_chunks = sort_chunks(a.cap);
    p.chunk_counts = bv.chunk_counts;
    p.digit_totals = bv.totals + kSortDigits * pass;
    int s = launch_pass(p, st);
    if (s != CFGS_OK) return s;
    src = dst;
  }
  k_tile_ranges<<<1, 1024, 0, st>>>(a.tile_count, a.tile_range, a.num_tiles);
  return CFGS_OK;
}
template int launch_binning<SingleScene>(const BinArgs<SingleScene>&, cudaStream_t);
template int launch_binning<SceneTable>(const BinArgs<SceneTable>&, cudaStream_t);

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
  BinArgs<SingleScene> a;
  a.scenes.d = single_scene_desc(s, g->num_gaussians, g->sh_coeffs);
  a.total_slots = g->num_gaussians;
  a.geom = GeomView(geom, g->num_gaussians);
  a.bin = BinningView(binning, capacity);
  a.cap = capacity;
  a.counts = iv.counts;
  a.num_tiles = IL.num_tiles;
  a.tile_count = iv.tile_count;
  a.tile_range = iv.tile_range;
  int status = launch_binning(a, st);
  if (status != CFGS_OK) return status;
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" void cfgs_binning_layout(int64_t cap, size_t o[8]) {
  BinningLayout L(cap);
  size_t v[8] = {L.key, L.gid, L.pidx, L.sorted_gid, L.sorted_pidx, L.chunk_counts, L.totals, L.total};
  for (int i = 0; i < 8; ++i) o[i] = v[i];
}
