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
// equal digits find each other with one ballot per digit bit.
#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kMaxDigitBits = 8;

// One radix pass over elements [0, n) split into chunks of `chunk` elements. Keys come
// from key_in, or (depth mode) from the geometry: the depth bits of Gaussians that
// touch a tile, ~0 for the others, so they sort last. Payloads come from val_in /
// aux_in, or are the element's own index when those are NULL.
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
  uint32_t* digit_totals;      // [1 << bits], written by the scan
};

__device__ __forceinline__ uint32_t pass_elements(const SortPass& p) {
  if (!p.counts) return (uint32_t)p.n;
  const int64_t k = (int64_t)p.counts->num_rendered;
  return k > p.cap ? 0u : (uint32_t)k;
}

// Loads the keys of elements [c0 + 4 j, c0 + 4 j + 4) (those below n) with one vector
// load where the four are in range.
template <bool DEPTH>
__device__ __forceinline__ uint4 load_keys4(const SortPass& p, uint32_t i, uint32_t n) {
  uint4 k = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
  if (DEPTH) {
    uint32_t* kk = &k.x;
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (i + e < n) kk[e] = p.depth_touched[i + e] ? __float_as_uint(p.depth_rgbd[i + e].w) : 0xffffffffu;
  } else if (i + 3 < n) {
    k = *reinterpret_cast<const uint4*>(p.key_in + i);
  } else {
    uint32_t* kk = &k.x;
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (i + e < n) kk[e] = p.key_in[i + e];
  }
  return k;
}

__device__ __forceinline__ uint4 load_u32x4(const uint32_t* a, uint32_t i, uint32_t n) {
  if (i + 3 < n) return *reinterpret_cast<const uint4*>(a + i);
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  uint32_t* vv = &v.x;
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (i + e < n) vv[e] = a[i + e];
  return v;
}

// Lanes of `active` whose digit equals this lane's: one ballot per digit bit. Every
// lane of the warp must call it.
__device__ __forceinline__ unsigned digit_peers(uint32_t d, int bits, unsigned active) {
  unsigned peers = active;
#pragma unroll
  for (int b = 0; b < kMaxDigitBits; ++b) {
    if (b < bits) {
      const bool set = (d >> b) & 1u;
      const unsigned bal = __ballot_sync(0xffffffffu, set);
      peers &= set ? bal : ~bal;
    }
  }
  return peers;
}

// Digit histogram of one chunk (per-warp shared-memory counters), written to
// chunk_counts[d][chunk].
template <int CHUNK, bool DEPTH>
__device__ __forceinline__ void sort_count_block(const SortPass& p, uint32_t bid) {
  __shared__ uint32_t hist[kSortWarps][kSortDigits];
  const uint32_t n = pass_elements(p);
  const uint32_t c0 = bid * (uint32_t)CHUNK;
  if (c0 >= n) return;
  const int ndig = 1 << p.bits;
  const uint32_t mask = (uint32_t)ndig - 1u;
  const int warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kSortWarps * kSortDigits; i += kSortThreads) (&hist[0][0])[i] = 0u;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < CHUNK / (4 * kSortThreads); ++k) {
    const uint32_t i = c0 + 4u * (k * kSortThreads + threadIdx.x);
    if (i < n) {
      const uint4 kk = load_keys4<DEPTH>(p, i, n);
      atomicAdd(&hist[warp][(kk.x >> p.shift) & mask], 1u);
      if (i + 1 < n) atomicAdd(&hist[warp][(kk.y >> p.shift) & mask], 1u);
      if (i + 2 < n) atomicAdd(&hist[warp][(kk.z >> p.shift) & mask], 1u);
      if (i + 3 < n) atomicAdd(&hist[warp][(kk.w >> p.shift) & mask], 1u);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < ndig; d += kSortThreads) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) s += hist[w][d];
    p.chunk_counts[(size_t)d * p.num_chunks + bid] = s;
  }
}
template <int CHUNK, bool DEPTH>
__global__ void __launch_bounds__(kSortThreads) k_sort_count(SortPass p) {
  sort_count_block<CHUNK, DEPTH>(p, blockIdx.x);
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

// One block per digit d: chunk_counts[d][c] becomes the number of digit-d elements in
// earlier chunks, and digit_totals[d] the digit's count. The scatter adds the counts of
// the smaller digits.
template <int CHUNK>
__device__ __forceinline__ void sort_scan_block(const SortPass& p, int d) {
  __shared__ uint32_t sh[64];
  const uint32_t n = pass_elements(p);
  const int64_t nc = ((int64_t)n + CHUNK - 1) / CHUNK;
  uint32_t tot, carry = 0;
  uint32_t* col = p.chunk_counts + (size_t)d * p.num_chunks;
  for (int64_t c0 = 0; c0 < nc; c0 += blockDim.x) {
    const int64_t c = c0 + threadIdx.x;
    const uint32_t v = c < nc ? col[c] : 0u;
    const uint32_t incl = block_inclusive_scan(v, sh, &tot);
    if (c < nc) col[c] = carry + incl - v;
    carry += tot;
  }
  if (threadIdx.x == 0) p.digit_totals[d] = carry;
}
template <int CHUNK>
__global__ void __launch_bounds__(1024) k_sort_scan(SortPass p) {
  sort_scan_block<CHUNK>(p, blockIdx.x);
}

// Shared memory of the scatter: keys and payloads in input order, the permutation
// (sorted position -> input position), per-warp digit counters, per-digit block-local
// starts and global slots.
template <int CHUNK>
struct ScatterSmem {
  static constexpr size_t kKey = 0;
  static constexpr size_t kVal = kKey + 4 * CHUNK;
  static constexpr size_t kAux = kVal + 4 * CHUNK;
  __host__ __device__ static size_t perm(bool aux) { return kAux + (aux ? 4 * CHUNK : 0); }
  __host__ __device__ static size_t whist(bool aux) { return perm(aux) + 2 * CHUNK; }
  __host__ __device__ static size_t start(bool aux) { return whist(aux) + 4 * kSortWarps * kSortDigits; }
  __host__ __device__ static size_t slot(bool aux) { return start(aux) + 4 * kSortDigits; }
  __host__ __device__ static size_t bytes(bool aux) { return slot(aux) + 4 * kSortDigits; }
};

template <int CHUNK, bool DEPTH>
__device__ __forceinline__ void sort_scatter_block(const SortPass& p, uint32_t bid) {
  using L = ScatterSmem<CHUNK>;
  constexpr int kSlice = CHUNK / kSortWarps;  // elements per warp
  constexpr int kRounds = kSlice / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const bool has_val = p.val_in != nullptr, has_aux = p.aux_in != nullptr;
  uint32_t* s_key = reinterpret_cast<uint32_t*>(smem_raw + L::kKey);
  uint32_t* s_val = reinterpret_cast<uint32_t*>(smem_raw + L::kVal);
  uint32_t* s_aux = reinterpret_cast<uint32_t*>(smem_raw + L::kAux);
  uint16_t* s_perm = reinterpret_cast<uint16_t*>(smem_raw + L::perm(has_aux));
  uint32_t* s_whist = reinterpret_cast<uint32_t*>(smem_raw + L::whist(has_aux));  // [warp][digit]
  uint32_t* s_start = reinterpret_cast<uint32_t*>(smem_raw + L::start(has_aux));
  uint32_t* s_slot = reinterpret_cast<uint32_t*>(smem_raw + L::slot(has_aux));
  __shared__ uint32_t sh[64];

  const uint32_t n = pass_elements(p);
  const uint32_t c0 = bid * (uint32_t)CHUNK;
  if (c0 >= n) return;
  const int cnt = (int)min((uint32_t)CHUNK, n - c0);
  const int ndig = 1 << p.bits;
  const uint32_t mask = (uint32_t)ndig - 1u;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

  // input chunk -> shared memory (vector loads, all in flight together)
#pragma unroll
  for (int k = 0; k < CHUNK / (4 * kSortThreads); ++k) {
    const int j = 4 * (k * kSortThreads + t);
    const uint32_t i = c0 + (uint32_t)j;
    if (i < n) {
      *reinterpret_cast<uint4*>(s_key + j) = load_keys4<DEPTH>(p, i, n);
      if (has_val) *reinterpret_cast<uint4*>(s_val + j) = load_u32x4(p.val_in, i, n);
      if (has_aux) *reinterpret_cast<uint4*>(s_aux + j) = load_u32x4(p.aux_in, i, n);
    }
  }
  for (int i = t; i < kSortWarps * kSortDigits; i += kSortThreads) s_whist[i] = 0u;
  __syncthreads();

  // rank of every element among the equal digits of its warp's slice
  uint32_t rank[kRounds];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < kRounds; ++k) {
    const int i = warp * kSlice + k * 32 + lane;
    const bool act = i < cnt;
    const unsigned am = __ballot_sync(0xffffffffu, act);
    const uint32_t d = act ? (s_key[i] >> p.shift) & mask : 0u;
    const unsigned peers = digit_peers(d, p.bits, am);
    const uint32_t before = act ? s_whist[warp * kSortDigits + d] : 0u;
    rank[k] = before + (uint32_t)__popc(peers & lt);
    __syncwarp();
    if (act && (peers & lt) == 0) s_whist[warp * kSortDigits + d] = before + (uint32_t)__popc(peers);
    __syncwarp();
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
  const uint32_t dtot = t < ndig ? p.digit_totals[t] : 0u;
  const uint32_t below = block_inclusive_scan(dtot, sh, &tot) - dtot;  // elements of smaller digits
  if (t < ndig) {
    s_start[t] = incl - dsum;
    s_slot[t] = dsum ? below + p.chunk_counts[(size_t)t * p.num_chunks + bid] : 0u;
  }
  __syncthreads();

  // permutation: block-local sorted position -> input position
#pragma unroll
  for (int k = 0; k < kRounds; ++k) {
    const int i = warp * kSlice + k * 32 + lane;
    if (i < cnt) {
      const uint32_t d = (s_key[i] >> p.shift) & mask;
      s_perm[s_start[d] + s_whist[warp * kSortDigits + d] + rank[k]] = (uint16_t)i;
    }
  }
  __syncthreads();

  // each digit's run goes to consecutive global slots
  for (int q = t; q < cnt; q += kSortThreads) {
    const int o = s_perm[q];
    const uint32_t kk = s_key[o];
    const uint32_t d = (kk >> p.shift) & mask;
    const uint32_t g = s_slot[d] + (uint32_t)q - s_start[d];
    if (p.key_out) p.key_out[g] = kk;
    p.val_out[g] = has_val ? s_val[o] : c0 + (uint32_t)o;
    if (p.aux_out) p.aux_out[g] = has_aux ? s_aux[o] : c0 + (uint32_t)o;
    if (p.tile_count) {
      // The chunk is fully sorted now (its input was sorted by the lower digits), so
      // equal tiles form runs: a run [b, e) adds e - b.
      if (q == 0 || s_key[s_perm[q - 1]] != kk) atomicSub(&p.tile_count[kk], (uint32_t)q);
      if (q == cnt - 1 || s_key[s_perm[q + 1]] != kk) atomicAdd(&p.tile_count[kk], (uint32_t)(q + 1));
    }
  }
}
template <int CHUNK, bool DEPTH>
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(SortPass p) {
  sort_scatter_block<CHUNK, DEPTH>(p, blockIdx.x);
}

// Instances of every 256 depth-ordered Gaussians (the emission's block prefix).
__device__ __forceinline__ void rank_sums_block(const uint32_t* order, const uint32_t* touched, int64_t total_slots,
                                                uint32_t* rank_sums, int bid) {
  __shared__ uint32_t sh[64];
  const int64_t r = (int64_t)bid * blockDim.x + threadIdx.x;
  const uint32_t v = r < total_slots ? touched[order[r]] : 0u;
  uint32_t tot;
  block_inclusive_scan(v, sh, &tot);
  if (threadIdx.x == 0) rank_sums[bid] = tot;
}
__global__ void __launch_bounds__(kPreprocessBlock) k_rank_sums(const uint32_t* order, const uint32_t* touched,
                                                                int64_t total_slots, uint32_t* rank_sums) {
  rank_sums_block(order, touched, total_slots, rank_sums, blockIdx.x);
}

// The per-block instance counts become their exclusive prefix, in place (one block): the
// emission's first instance index of each block of 256 depth-ordered Gaussians. Run for
// large batches only: below kRankScanMinBlocks blocks each emission block sums its
// predecessors itself (cheaper than a launch; quadratic in the block count above it).
constexpr int kRankScanMinBlocks = 8192;
inline bool rank_scan_needed(int rank_blocks) { return rank_blocks > kRankScanMinBlocks; }
__device__ __forceinline__ void rank_scan_block(uint32_t* rank_sums, int n) {
  __shared__ uint32_t sh[64];
  uint32_t carry = 0, tot;
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    const uint32_t v = c < n ? rank_sums[c] : 0u;
    const uint32_t incl = block_inclusive_scan(v, sh, &tot);
    if (c < n) rank_sums[c] = carry + incl - v;
    carry += tot;
  }
}
__global__ void __launch_bounds__(1024) k_rank_scan(uint32_t* rank_sums, int n) { rank_scan_block(rank_sums, n); }

// One thread per depth-ordered Gaussian; the block's first instance index is the sum of
// the earlier blocks' rank_sums (formed by k_rank_scan for large batches, else by the
// block itself), the thread's is that plus a block scan. The
// instances are then written warp-cooperatively: the warp's instances are dealt out
// 32 per round, one per lane, so the stores of a round are consecutive. In a round, the
// lanes whose instance ranges meet it mark where their range begins (an OR reduction),
// and a lane's owner is the last mark at or before it; the owner's rectangle comes over
// by shuffle. Instance j of a rectangle of width w is tile row j / w, column j % w; the
// quotient is estimated with a float reciprocal (off by at most one for j < 2^22) and
// corrected exactly.
template <class Scenes>
__device__ __forceinline__ void emit_block(const EmitArgs<Scenes>& a, int bid) {
  __shared__ uint32_t sh[64];
  __shared__ uint8_t s_owner[kPreprocessBlock / 32][32];
  if ((int64_t)a.counts->num_rendered > a.cap) {
    if (bid == 0 && threadIdx.x == 0) atomicOr(&a.counts->flags, CFGS_FLAG_CAPACITY_OVERFLOW);
    return;
  }
  uint32_t tot, block_first;
  if (a.rank_scanned) {
    block_first = a.rank_sums[bid];  // exclusive prefix (k_rank_scan)
  } else {
    uint32_t pre = 0;
#pragma unroll 4
    for (int b = threadIdx.x; b < bid; b += blockDim.x) pre += a.rank_sums[b];
    block_inclusive_scan(pre, sh, &tot);
    block_first = tot;
  }
  const int64_t r = (int64_t)bid * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t g = 0, nt = 0;
  if (r < a.total_slots) {
    g = a.order[r];
    nt = a.geom.touched[g];
  }
  const uint32_t first = block_first + block_inclusive_scan(nt, sh, &tot) - nt;
  uint2 rc = make_uint2(0u, 0u);
  uint32_t tile_base = 0, grid_x = 0;
  float rinv = 0.0f;
  if (nt) {
    a.geom.offset[g] = first;
    const SceneDesc& sd = a.scenes.for_gaussian(g);
    rc = a.geom.rect[g];
    tile_base = (uint32_t)sd.tile_base;
    grid_x = (uint32_t)sd.grid_x;
    rinv = 1.0f / (float)((rc.y & 0xffffu) - (rc.x & 0xffffu));
  }
  // warp-exclusive start of this lane's instances
  uint32_t x = nt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const uint32_t warp_total = __shfl_sync(0xffffffffu, x, 31);
  const uint32_t start = x - nt;
  const unsigned upto = 0xffffffffu >> (31 - lane);  // bits 0..lane
  for (uint32_t base = 0; base < warp_total; base += 32) {
    const bool meets = nt != 0 && start < base + 32u && start + nt > base;
    const uint32_t pos = start > base ? start - base : 0u;
    const unsigned marks = __reduce_or_sync(0xffffffffu, meets ? (1u << pos) : 0u);
    if (meets) s_owner[warp][pos] = (uint8_t)lane;
    __syncwarp();
    const int o = s_owner[warp][31 - __clz(marks & upto)];
    __syncwarp();
    const uint32_t o_start = __shfl_sync(0xffffffffu, start, o);
    const uint32_t o_rx = __shfl_sync(0xffffffffu, rc.x, o);
    const uint32_t o_ry = __shfl_sync(0xffffffffu, rc.y, o);
    const uint32_t o_first = __shfl_sync(0xffffffffu, first, o);
    const uint32_t o_gid = __shfl_sync(0xffffffffu, g, o);
    const float o_rinv = __shfl_sync(0xffffffffu, rinv, o);
    const uint32_t o_tb = __shfl_sync(0xffffffffu, tile_base, o);
    const uint32_t o_gx = __shfl_sync(0xffffffffu, grid_x, o);
    const uint32_t w = base + (uint32_t)lane;
    if (w < warp_total) {
      const uint32_t j = w - o_start;
      const uint32_t x0 = o_rx & 0xffffu, y0 = o_rx >> 16;
      const uint32_t rw = (o_ry & 0xffffu) - x0;
      uint32_t ty, tx;
      if (j < (1u << 22)) {
        ty = (uint32_t)((float)j * o_rinv);
        tx = j - ty * rw;
        if ((int32_t)tx < 0) {
          --ty;
          tx += rw;
        } else if (tx >= rw) {
          ++ty;
          tx -= rw;
        }
      } else {
        ty = j / rw;
        tx = j - ty * rw;
      }
      const uint32_t q = o_first + j;
      a.bin.key[0][q] = o_tb + (y0 + ty) * o_gx + x0 + tx;
      a.bin.gid[0][q] = o_gid;
    }
  }
}
template <class Scenes>
__global__ void __launch_bounds__(kPreprocessBlock) k_emit(EmitArgs<Scenes> a) {
  emit_block<Scenes>(a, blockIdx.x);
}

// Tile ranges from the per-tile instance counts (one block).
__device__ __forceinline__ void tile_ranges_block(const uint32_t* tile_count, uint32_t* tile_range, int num_tiles) {
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
__global__ void __launch_bounds__(1024) k_tile_ranges(const uint32_t* tile_count, uint32_t* tile_range, int num_tiles) {
  tile_ranges_block(tile_count, tile_range, num_tiles);
}

namespace {

template <int CHUNK, bool DEPTH>
int launch_pass(const SortPass& p, cudaStream_t st) {
  static std::atomic<uint64_t> smem_set{0};
  if (!ensure_dynamic_smem(k_sort_scatter<CHUNK, DEPTH>, (int)ScatterSmem<CHUNK>::bytes(true), smem_set))
    return CFGS_ERR_LAUNCH;
  const int grid = (int)p.num_chunks;
  k_sort_count<CHUNK, DEPTH><<<grid, kSortThreads, 0, st>>>(p);
  k_sort_scan<CHUNK><<<1 << p.bits, 1024, 0, st>>>(p);
  k_sort_scatter<CHUNK, DEPTH>
      <<<grid, kSortThreads, ScatterSmem<CHUNK>::bytes(p.aux_in != nullptr), st>>>(p);
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

// Step 1 of the binning, which needs no instance capacity: the depth order of the
// Gaussians and their instance counts per 256 in that order.
int launch_depth_order(const GeomView& gv, int64_t slots, cudaStream_t st) {
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
      p.num_chunks = sort_chunks(slots, kDepthChunk);
      p.chunk_counts = gv.depth_counts;
      p.digit_totals = gv.depth_totals + kSortDigits * pass;
      int s = src < 0 ? launch_pass<kDepthChunk, true>(p, st) : launch_pass<kDepthChunk, false>(p, st);
      if (s != CFGS_OK) return s;
      src = dst;
    }
    const int rank_blocks = (int)((slots + kPreprocessBlock - 1) / kPreprocessBlock);
    k_rank_sums<<<rank_blocks, kPreprocessBlock, 0, st>>>(gv.depth_val[1], gv.touched, slots, gv.rank_sums);
    if (rank_scan_needed(rank_blocks)) k_rank_scan<<<1, 1024, 0, st>>>(gv.rank_sums, rank_blocks);
  }
  return CFGS_OK;
}

// Steps 2-3, after launch_depth_order: emission in depth order, tile sort, tile ranges.
template <class Scenes>
int launch_instances(const BinArgs<Scenes>& a, cudaStream_t st) {
  const GeomView& gv = a.geom;
  const BinningView& bv = a.bin;
  const int64_t slots = a.total_slots;
  if (slots > 0) {
    // 2. emission in depth order
    const int rank_blocks = (int)((slots + kPreprocessBlock - 1) / kPreprocessBlock);
    EmitArgs<Scenes> e;
    e.scenes = a.scenes;
    e.total_slots = slots;
    e.order = gv.depth_val[1];
    e.rank_sums = gv.rank_sums;
    e.rank_scanned = rank_scan_needed(rank_blocks);
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
    p.num_chunks = sort_chunks(a.cap, kTileChunk);
    p.chunk_counts = bv.chunk_counts;
    p.digit_totals = bv.totals + kSortDigits * pass;
    int s = launch_pass<kTileChunk, false>(p, st);
    if (s != CFGS_OK) return s;
    src = dst;
  }
  k_tile_ranges<<<1, 1024, 0, st>>>(a.tile_count, a.tile_range, a.num_tiles);
  return CFGS_OK;
}

// ---- the binning as one persistent launch ----------------------------------------------
// The same block functions as the per-stage kernels above, run by a cooperative grid of
// resident 256-thread blocks: each stage's blocks are dealt out over the grid, and a
// bounded grid-wide wait separates the stages (each reads what the previous one wrote).
// The outputs are the per-stage launches' outputs (integer work, same order).
template <class Scenes>
struct PersistentBinArgs {
  SortPass depth[kDepthPasses];
  const uint32_t* order;
  const uint32_t* touched;
  int64_t slots;
  uint32_t* rank_sums;
  int rank_blocks;
  EmitArgs<Scenes> emit;
  SortPass tile[kMaxTilePasses];
  int tile_passes;
  const uint32_t* tile_count;
  uint32_t* tile_range;
  int num_tiles;
  GridBarrier* barrier;
  uint32_t* flags;
};

template <class Scenes>
__global__ void __launch_bounds__(kSortThreads) k_binning_persistent(PersistentBinArgs<Scenes> a) {
  static_assert(kSortThreads == kPreprocessBlock && kDepthChunk == kTileChunk, "one block shape for every stage");
  auto each = [&](int64_t blocks, auto&& block_fn) {
    for (int64_t b = blockIdx.x; b < blocks; b += gridDim.x) {
      block_fn((uint32_t)b);
      __syncthreads();  // the block's shared memory is reused by its next virtual block
    }
  };
  for (int pass = 0; pass < kDepthPasses; ++pass) {
    const SortPass& p = a.depth[pass];
    if (pass == 0) each(p.num_chunks, [&](uint32_t b) { sort_count_block<kDepthChunk, true>(p, b); });
    else each(p.num_chunks, [&](uint32_t b) { sort_count_block<kDepthChunk, false>(p, b); });
    if (!grid_barrier(a.barrier, a.flags)) return;
    each(1 << p.bits, [&](uint32_t b) { sort_scan_block<kDepthChunk>(p, (int)b); });
    if (!grid_barrier(a.barrier, a.flags)) return;
    if (pass == 0) each(p.num_chunks, [&](uint32_t b) { sort_scatter_block<kDepthChunk, true>(p, b); });
    else each(p.num_chunks, [&](uint32_t b) { sort_scatter_block<kDepthChunk, false>(p, b); });
    if (!grid_barrier(a.barrier, a.flags)) return;
  }
  each(a.rank_blocks, [&](uint32_t b) { rank_sums_block(a.order, a.touched, a.slots, a.rank_sums, (int)b); });
  if (!grid_barrier(a.barrier, a.flags)) return;
  if (a.emit.rank_scanned) {
    if (blockIdx.x == 0) rank_scan_block(a.rank_sums, a.rank_blocks);
    if (!grid_barrier(a.barrier, a.flags)) return;
  }
  each(a.rank_blocks, [&](uint32_t b) { emit_block<Scenes>(a.emit, (int)b); });
  if (!grid_barrier(a.barrier, a.flags)) return;
  for (int pass = 0; pass < a.tile_passes; ++pass) {
    const SortPass& p = a.tile[pass];
    each(p.num_chunks, [&](uint32_t b) { sort_count_block<kTileChunk, false>(p, b); });
    if (!grid_barrier(a.barrier, a.flags)) return;
    each(1 << p.bits, [&](uint32_t b) { sort_scan_block<kTileChunk>(p, (int)b); });
    if (!grid_barrier(a.barrier, a.flags)) return;
    each(p.num_chunks, [&](uint32_t b) { sort_scatter_block<kTileChunk, false>(p, b); });
    if (!grid_barrier(a.barrier, a.flags)) return;
  }
  if (blockIdx.x == 0) tile_ranges_block(a.tile_count, a.tile_range, a.num_tiles);
}

// The pass descriptions of launch_depth_order and launch_instances, for one launch.
template <class Scenes>
int launch_binning_persistent(const BinArgs<Scenes>& a, GridBarrier* barrier, cudaStream_t st) {
  const GeomView& gv = a.geom;
  const BinningView& bv = a.bin;
  const int64_t slots = a.total_slots;
  if (slots <= 0) return launch_instances(a, st);
  PersistentBinArgs<Scenes> pa{};
  int src = -1;
  for (int pass = 0; pass < kDepthPasses; ++pass) {
    SortPass& p = pa.depth[pass];
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
    p.num_chunks = sort_chunks(slots, kDepthChunk);
    p.chunk_counts = gv.depth_counts;
    p.digit_totals = gv.depth_totals + kSortDigits * pass;
    src = dst;
  }
  const int rank_blocks = (int)((slots + kPreprocessBlock - 1) / kPreprocessBlock);
  pa.order = gv.depth_val[1];
  pa.touched = gv.touched;
  pa.slots = slots;
  pa.rank_sums = gv.rank_sums;
  pa.rank_blocks = rank_blocks;
  EmitArgs<Scenes>& e = pa.emit;
  e.scenes = a.scenes;
  e.total_slots = slots;
  e.order = gv.depth_val[1];
  e.rank_sums = gv.rank_sums;
  e.rank_scanned = rank_scan_needed(rank_blocks);
  e.geom = gv;
  e.bin = bv;
  e.cap = a.cap;
  e.counts = a.counts;
  int passes, width;
  tile_sort_plan(a.num_tiles, &passes, &width);
  if (passes > kMaxTilePasses) return CFGS_ERR_TOO_LARGE;
  pa.tile_passes = passes;
  src = 0;
  for (int pass = 0; pass < passes; ++pass) {
    SortPass& p = pa.tile[pass];
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
    p.num_chunks = sort_chunks(a.cap, kTileChunk);
    p.chunk_counts = bv.chunk_counts;
    p.digit_totals = bv.totals + kSortDigits * pass;
    src = dst;
  }
  pa.tile_count = a.tile_count;
  pa.tile_range = a.tile_range;
  pa.num_tiles = (int)a.num_tiles;
  pa.barrier = barrier;
  pa.flags = &a.counts->flags;

  // every block resident: the grid is the kernel's occupancy times the SM count (per device)
  const int smem = (int)ScatterSmem<kTileChunk>::bytes(true);
  static std::atomic<uint64_t> smem_set{0};
  if (!ensure_dynamic_smem(k_binning_persistent<Scenes>, smem, smem_set)) return CFGS_ERR_LAUNCH;
  static std::atomic<int> grid_of_device[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CFGS_ERR_LAUNCH;
  int grid = dev < 64 ? grid_of_device[dev].load(std::memory_order_acquire) : 0;
  if (grid <= 0) {
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_binning_persistent<Scenes>, kSortThreads, smem) !=
            cudaSuccess ||
        sms <= 0 || per_sm <= 0)
      return CFGS_ERR_LAUNCH;
    grid = sms * per_sm;
    if (dev < 64) grid_of_device[dev].store(grid, std::memory_order_release);
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kSortThreads);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, k_binning_persistent<Scenes>, pa) != cudaSuccess) return CFGS_ERR_LAUNCH;
  return CFGS_OK;
}
template int launch_binning_persistent<SceneTable>(const BinArgs<SceneTable>&, GridBarrier*, cudaStream_t);

template <class Scenes>
int launch_binning(const BinArgs<Scenes>& a, cudaStream_t st) {
  const int s = launch_depth_order(a.geom, a.total_slots, st);
  return s != CFGS_OK ? s : launch_instances(a, st);
}
template int launch_binning<SingleScene>(const BinArgs<SingleScene>&, cudaStream_t);

// Stable LSD radix sort of n (key, value) pairs by the low `bits` key bits, passes of at
// most 8 bits, ping-ponging between (keys[0], vals[0]) and (keys[1], vals[1]); returns
// the index (0 or 1) of the buffers holding the result. chunk_counts holds
// 256 x sort_chunks(n, kTileChunk) values, totals 256 x kMaxTilePasses.
int sort_pairs(uint32_t* keys[2], uint32_t* vals[2], int64_t n, int bits, uint32_t* chunk_counts, uint32_t* totals,
               cudaStream_t st, int* result) {
  if (bits < 1 || bits > 32 || n < 0 || n > 0x7fffffffll) return CFGS_ERR_INVALID_ARGUMENT;
  const int passes = (bits + 7) / 8;
  const int width = (bits + passes - 1) / passes;
  int src = 0;
  for (int pass = 0; pass < passes; ++pass) {
    SortPass p{};
    const int dst = src ^ 1;
    p.key_in = keys[src];
    p.val_in = vals[src];
    p.key_out = keys[dst];
    p.val_out = vals[dst];
    p.shift = width * pass;
    p.bits = min(width, bits - width * pass);
    p.n = n;
    p.cap = n;
    p.num_chunks = sort_chunks(n, kTileChunk);
    p.chunk_counts = chunk_counts;
    p.digit_totals = totals + kSortDigits * pass;
    int s = launch_pass<kTileChunk, false>(p, st);
    if (s != CFGS_OK) return s;
    src = dst;
  }
  *result = src;
  return CFGS_OK;
}

template int launch_binning<SceneTable>(const BinArgs<SceneTable>&, cudaStream_t);

}  // namespace cfgs

using namespace cfgs;

namespace {

// The single-scene binning arguments of the drop-in path.
int single_bin_args(const CfgsSettings* s, const CfgsGaussians* g, void* geom, void* image, void* binning,
                    int64_t capacity, BinArgs<SingleScene>* a) {
  if (!s || !g || !geom || !image || !binning || capacity < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (s->image_width <= 0 || s->image_height <= 0 || g->num_gaussians < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity > 0x7fffffffll) return CFGS_ERR_TOO_LARGE;
  ImageLayout IL(s->image_width, s->image_height);
  ImageView iv(image, s->image_width, s->image_height);
  a->scenes.d = single_scene_desc(s, g->num_gaussians, g->sh_coeffs);
  a->total_slots = g->num_gaussians;
  a->geom = GeomView(geom, g->num_gaussians);
  a->bin = BinningView(binning, capacity);
  a->cap = capacity;
  a->counts = iv.counts;
  a->num_tiles = IL.num_tiles;
  a->tile_count = iv.tile_count;
  a->tile_range = iv.tile_range;
  return CFGS_OK;
}

}  // namespace

extern "C" int cfgs_bin_forward(const CfgsSettings* s, const CfgsGaussians* g, void* geom, void* image, void* binning,
                                int64_t capacity, void* stream) {
  BinArgs<SingleScene> a;
  int status = single_bin_args(s, g, geom, image, binning, capacity, &a);
  if (status != CFGS_OK) return status;
  cudaStream_t st = (cudaStream_t)stream;
  status = launch_binning(a, st);
  if (status != CFGS_OK) return status;
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_depth_order(int32_t num_gaussians, void* geom, void* stream) {
  if (num_gaussians < 0 || (num_gaussians > 0 && !geom)) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  const int status = launch_depth_order(GeomView(geom, num_gaussians), num_gaussians, st);
  if (status != CFGS_OK) return status;
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}

extern "C" int cfgs_bin_instances(const CfgsSettings* s, const CfgsGaussians* g, void* geom, void* image,
                                  void* binning, int64_t capacity, void* stream) {
  BinArgs<SingleScene> a;
  int status = single_bin_args(s, g, geom, image, binning, capacity, &a);
  if (status != CFGS_OK) return status;
  cudaStream_t st = (cudaStream_t)stream;
  status = launch_instances(a, st);
  if (status != CFGS_OK) return status;
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" void cfgs_binning_layout(int64_t cap, size_t o[8]) {
  BinningLayout L(cap);
  size_t v[8] = {L.key, L.gid, L.pidx, L.sorted_gid, L.sorted_pidx, L.chunk_counts, L.totals, L.total};
  for (int i = 0; i < 8; ++i) o[i] = v[i];
}
