// Internal definitions shared by the rasteriser translation units: workspace
// layouts, launch helpers and the scalar math whose rounding the CPU oracle mirrors.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/cfgs.h"

namespace cfgs {

constexpr int kTileX = CFGS_TILE_X;
constexpr int kTileY = CFGS_TILE_Y;
constexpr int kTilePixels = kTileX * kTileY;  // 256
constexpr int kPreprocessBlock = 256;
constexpr int kMaxShCoeffs = 16;  // SH degree 3
#define CFGS_SH_BULK_COEFFS 16

// ---------------------------------------------------------------------------
// Workspace layouts. Every array starts on a 256-byte boundary.
// ---------------------------------------------------------------------------
__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Raises a kernel's dynamic shared-memory limit to `bytes` on the current device, once
// per device (a function attribute belongs to the device's context, so one flag per
// process would leave a second GPU of the process without it). `done` is the kernel's
// own set of device bits; devices past 63 set the attribute on every call.
template <class Kernel>
inline bool ensure_dynamic_smem(Kernel* kernel, int bytes, std::atomic<uint64_t>& done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  const uint64_t bit = dev < 64 ? (uint64_t)1 << dev : 0;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return true;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return false;
  done.fetch_or(bit, std::memory_order_acq_rel);
  return true;
}

// Binning sorts (stable LSD radix, at most 8 bits per pass) work on chunks of
// elements: kDepthChunk for the depth sort of the Gaussians (4 passes), kTileChunk for
// the tile sort of the instances.
constexpr int kDepthChunk = 1024;
constexpr int kTileChunk = 1024;
constexpr int kSortDigits = 256;  // digits per pass at most (8 bits)
constexpr int kDepthPasses = 4;
constexpr int kMaxTilePasses = 4;

__host__ __device__ inline int64_t sort_chunks(int64_t n, int chunk) { return n > 0 ? (n + chunk - 1) / chunk : 1; }
// Element stride of the halves of a ping-pong sort buffer: a multiple of 64 elements, so
// both halves start on a 256-byte boundary (the sort passes use 16-byte vector loads).
__host__ __device__ inline size_t pingpong_stride(int64_t n) { return ((size_t)(n > 0 ? n : 1) + 63) & ~size_t(63); }

struct GeomLayout {
  size_t xy, conic_op, rgbd, rect, touched, offset, clamped, block_sums, depth_key, depth_val, rank_sums,
      depth_counts, depth_totals, total;
  int32_t num_blocks;
  __host__ __device__ explicit GeomLayout(int32_t n) {
    num_blocks = (n + kPreprocessBlock - 1) / kPreprocessBlock;
    const size_t sn = pingpong_stride(n);
    size_t o = 0;
    xy = o;           o = align256(o + sizeof(float) * 2 * (size_t)n);
    conic_op = o;     o = align256(o + sizeof(float) * 4 * (size_t)n);
    rgbd = o;         o = align256(o + sizeof(float) * 4 * (size_t)n);
    rect = o;         o = align256(o + sizeof(uint32_t) * 2 * (size_t)n);
    touched = o;      o = align256(o + sizeof(uint32_t) * (size_t)n);
    offset = o;       o = align256(o + sizeof(uint32_t) * (size_t)n);
    clamped = o;      o = align256(o + (size_t)n);
    block_sums = o;   o = align256(o + sizeof(uint32_t) * (size_t)(num_blocks + 1));
    depth_key = o;    o = align256(o + sizeof(uint32_t) * 2 * sn);
    depth_val = o;    o = align256(o + sizeof(uint32_t) * 2 * sn);
    rank_sums = o;    o = align256(o + sizeof(uint32_t) * (size_t)(num_blocks + 1));
    depth_counts = o; o = align256(o + sizeof(uint32_t) * kSortDigits * (size_t)sort_chunks(n, kDepthChunk));
    depth_totals = o; o = align256(o + sizeof(uint32_t) * kSortDigits * kDepthPasses);
    total = o;
  }
};

struct GeomView {
  float2* xy;          // pixel-space centre
  float4* conic_op;    // (conic a, conic b, conic c, opacity)
  float4* rgbd;        // (r, g, b, view depth)
  uint2* rect;         // (min_x | min_y << 16, max_x | max_y << 16) in tiles
  uint32_t* touched;   // tiles touched (0 = culled)
  uint32_t* offset;    // first instance index of the Gaussian (instances are numbered in depth order)
  uint8_t* clamped;    // bit c set: SH colour channel c was clamped at 0
  uint32_t* block_sums;
  uint32_t* depth_key[2];  // depth sort ping-pong keys
  uint32_t* depth_val[2];  // depth sort ping-pong Gaussian ids; depth_val[1] = Gaussians in depth order
  uint32_t* rank_sums;     // instances per 256 depth-ordered Gaussians
  uint32_t* depth_counts;  // [256][chunks] per-pass digit counts, then first slots
  uint32_t* depth_totals;  // [passes][256] digit totals
  __host__ __device__ GeomView() {}
  __host__ __device__ GeomView(void* base, int32_t n) {
    GeomLayout L(n);
    const size_t sn = pingpong_stride(n);
    char* b = static_cast<char*>(base);
    xy = reinterpret_cast<float2*>(b + L.xy);
    conic_op = reinterpret_cast<float4*>(b + L.conic_op);
    rgbd = reinterpret_cast<float4*>(b + L.rgbd);
    rect = reinterpret_cast<uint2*>(b + L.rect);
    touched = reinterpret_cast<uint32_t*>(b + L.touched);
    offset = reinterpret_cast<uint32_t*>(b + L.offset);
    clamped = reinterpret_cast<uint8_t*>(b + L.clamped);
    block_sums = reinterpret_cast<uint32_t*>(b + L.block_sums);
    depth_key[0] = reinterpret_cast<uint32_t*>(b + L.depth_key);
    depth_key[1] = depth_key[0] + sn;
    depth_val[0] = reinterpret_cast<uint32_t*>(b + L.depth_val);
    depth_val[1] = depth_val[0] + sn;
    rank_sums = reinterpret_cast<uint32_t*>(b + L.rank_sums);
    depth_counts = reinterpret_cast<uint32_t*>(b + L.depth_counts);
    depth_totals = reinterpret_cast<uint32_t*>(b + L.depth_totals);
  }
};

struct ImageLayout {
  size_t header, tile_count, tile_range, final_T, n_contrib, total;
  int32_t grid_x, grid_y, num_tiles;
  __host__ __device__ ImageLayout(int32_t w, int32_t h) {
    grid_x = (w + kTileX - 1) / kTileX;
    grid_y = (h + kTileY - 1) / kTileY;
    num_tiles = grid_x * grid_y;
    size_t px = (size_t)w * (size_t)h;
    size_t o = 0;
    header = o;      o = align256(o + sizeof(CfgsCounts));
    tile_count = o;  o = align256(o + sizeof(uint32_t) * (size_t)num_tiles);
    tile_range = o;  o = align256(o + sizeof(uint32_t) * (size_t)(num_tiles + 1));
    final_T = o;     o = align256(o + sizeof(float) * px);
    n_contrib = o;   o = align256(o + sizeof(uint32_t) * px);
    total = o;
  }
};

struct ImageView {
  CfgsCounts* counts;
  uint32_t* tile_count;
  uint32_t* tile_range;   // [num_tiles + 1]: tile t owns sorted positions [r[t], r[t+1])
  float* final_T;
  uint32_t* n_contrib;
  __host__ __device__ ImageView() {}
  __host__ __device__ ImageView(void* base, int32_t w, int32_t h) {
    ImageLayout L(w, h);
    char* b = static_cast<char*>(base);
    counts = reinterpret_cast<CfgsCounts*>(b + L.header);
    tile_count = reinterpret_cast<uint32_t*>(b + L.tile_count);
    tile_range = reinterpret_cast<uint32_t*>(b + L.tile_range);
    final_T = reinterpret_cast<float*>(b + L.final_T);
    n_contrib = reinterpret_cast<uint32_t*>(b + L.n_contrib);
  }
};

// Instances (one per Gaussian and touched tile). The emission writes them in depth
// order (tile key, Gaussian id; the instance index is the position); the tile sort
// passes ping-pong between the two buffers and the last one writes sorted_gid and
// sorted_pidx.
struct BinningLayout {
  size_t key, gid, pidx, sorted_gid, sorted_pidx, chunk_counts, totals, total;
  __host__ __device__ explicit BinningLayout(int64_t cap) {
    const size_t c = pingpong_stride(cap);
    size_t o = 0;
    key = o;          o = align256(o + sizeof(uint32_t) * 2 * c);
    gid = o;          o = align256(o + sizeof(uint32_t) * 2 * c);
    pidx = o;         o = align256(o + sizeof(uint32_t) * 2 * c);
    sorted_gid = o;   o = align256(o + sizeof(uint32_t) * c);
    sorted_pidx = o;  o = align256(o + sizeof(uint32_t) * c);
    chunk_counts = o; o = align256(o + sizeof(uint32_t) * kSortDigits * (size_t)sort_chunks(cap, kTileChunk));
    totals = o;       o = align256(o + sizeof(uint32_t) * kSortDigits * kMaxTilePasses);
    total = o;
  }
};

struct BinningView {
  uint32_t* key[2];       // global tile index of the instance
  uint32_t* gid[2];       // Gaussian id
  uint32_t* pidx[2];      // instance index (position in depth order)
  uint32_t* sorted_gid;   // sorted position -> Gaussian id
  uint32_t* sorted_pidx;  // sorted position -> instance index
  uint32_t* chunk_counts; // [256][chunks] per-pass digit counts, then first slots
  uint32_t* totals;       // [passes][256] digit totals
  __host__ __device__ BinningView() {}
  __host__ __device__ BinningView(void* base, int64_t cap) {
    BinningLayout L(cap);
    const size_t c = pingpong_stride(cap);
    char* b = static_cast<char*>(base);
    key[0] = reinterpret_cast<uint32_t*>(b + L.key);
    key[1] = key[0] + c;
    gid[0] = reinterpret_cast<uint32_t*>(b + L.gid);
    gid[1] = gid[0] + c;
    pidx[0] = reinterpret_cast<uint32_t*>(b + L.pidx);
    pidx[1] = pidx[0] + c;
    sorted_gid = reinterpret_cast<uint32_t*>(b + L.sorted_gid);
    sorted_pidx = reinterpret_cast<uint32_t*>(b + L.sorted_pidx);
    chunk_counts = reinterpret_cast<uint32_t*>(b + L.chunk_counts);
    totals = reinterpret_cast<uint32_t*>(b + L.totals);
  }
};

// ---------------------------------------------------------------------------
// Scenes. Every kernel reads its camera and image geometry through a scene
// accessor: SingleScene (the drop-in path: one descriptor passed by value) or
// SceneTable (batched solves: descriptors in device memory, looked up per block of
// Gaussians and per tile). The kernels' arithmetic is the same for both.
// Batched layout: scene s owns Gaussians [gauss_base, gauss_base + num_gaussians)
// with gauss_base a multiple of kPreprocessBlock (blocks never straddle scenes),
// tiles [tile_base, tile_base + num_tiles) and pixels [pix_base, pix_base + W*H);
// per-pixel images of scene s start at pix_base (3*pix_base for colour, channel-major
// inside the scene: [3, H, W]).
// ---------------------------------------------------------------------------
struct PoseState {     // per-scene rigid motion applied to the means before projection
  double R64[9];       // rotation of exp(xi), float64 (pose-gradient terms)
  double t64[3];
  double Jl[9];        // SO(3) left Jacobian of phi and the block Q(rho, phi) of the SE(3) one:
  double Q[9];         // dL/dxi = [[Jl, Q], [0, Jl]]^T dL/d(left perturbation)
  double bc1, bc2;     // Adam bias corrections 1 - beta^step of the step the solve takes next
  float R[9];          // the same, rounded to float (positions)
  float t[3];
};

struct SceneDesc {
  int32_t W, H, grid_x, grid_y;
  int32_t tile_base, num_tiles;
  int32_t gauss_base, num_gaussians;
  int64_t pix_base;
  int32_t sh_degree, sh_coeffs;
  int32_t prefiltered, pad_;
  float tanfovx, tanfovy, focal_x, focal_y, scale_modifier, inv_numel;
  const float* V;       // [16] world_view_transform
  const float* P;       // [16] full_proj_transform
  const float* campos;  // [3]
  const float* bg;      // [3]
  const PoseState* pose;  // NULL: means3D are used as given
};

struct SingleScene {
  static constexpr bool kBatched = false;
  SceneDesc d;
  __device__ __forceinline__ const SceneDesc& for_block(int) const { return d; }
  __device__ __forceinline__ const SceneDesc& for_tile(int) const { return d; }
  __device__ __forceinline__ const SceneDesc& for_gaussian(int64_t) const { return d; }
};

struct SceneTable {
  static constexpr bool kBatched = true;
  const SceneDesc* d;
  const int32_t* block_scene;  // preprocess block -> scene
  const int32_t* tile_scene;   // global tile -> scene
  __device__ __forceinline__ const SceneDesc& for_block(int b) const { return d[block_scene[b]]; }
  __device__ __forceinline__ const SceneDesc& for_tile(int t) const { return d[tile_scene[t]]; }
  __device__ __forceinline__ const SceneDesc& for_gaussian(int64_t g) const {
    return d[block_scene[g / kPreprocessBlock]];
  }
};

// Position of Gaussian i as the projection sees it: the stored mean, or R p + t in
// the order ((R0 x + R1 y) + R2 z) + t with one rounding per operation.
__device__ __forceinline__ float3 posed_mean(const SceneDesc& sd, const float* means, size_t i) {
  float3 p = make_float3(means[3 * i], means[3 * i + 1], means[3 * i + 2]);
  if (sd.pose == nullptr) return p;
  const float* R = sd.pose->R;
  const float* t = sd.pose->t;
  float3 q;
  q.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(R[0], p.x), __fmul_rn(R[1], p.y)), __fmul_rn(R[2], p.z)), t[0]);
  q.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(R[3], p.x), __fmul_rn(R[4], p.y)), __fmul_rn(R[5], p.z)), t[1]);
  q.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(R[6], p.x), __fmul_rn(R[7], p.y)), __fmul_rn(R[8], p.z)), t[2]);
  return q;
}

// Host helper: the descriptor of the drop-in path's single scene.
inline SceneDesc single_scene_desc(const CfgsSettings* s, int32_t n, int32_t sh_coeffs) {
  SceneDesc d{};
  d.W = s->image_width;
  d.H = s->image_height;
  d.grid_x = (d.W + kTileX - 1) / kTileX;
  d.grid_y = (d.H + kTileY - 1) / kTileY;
  d.tile_base = 0;
  d.num_tiles = d.grid_x * d.grid_y;
  d.gauss_base = 0;
  d.num_gaussians = n;
  d.pix_base = 0;
  d.sh_degree = s->sh_degree;
  d.sh_coeffs = sh_coeffs;
  d.prefiltered = s->prefiltered;
  d.tanfovx = s->tanfovx;
  d.tanfovy = s->tanfovy;
  d.focal_x = (float)s->image_width / (2.0f * s->tanfovx);
  d.focal_y = (float)s->image_height / (2.0f * s->tanfovy);
  d.scale_modifier = s->scale_modifier;
  d.inv_numel = 1.0f / (float)(3.0 * (double)d.W * (double)d.H);
  d.V = s->viewmatrix;
  d.P = s->projmatrix;
  d.campos = s->campos;
  d.bg = s->bg;
  d.pose = nullptr;
  return d;
}

// Backward scratch: one 48-byte record per pre-sort instance:
// (dxy.x, dxy.y, dconic.a, dconic.b) (dconic.c, dopacity, drgb.r, drgb.g) (drgb.b, ddepth, 0, 0)
// and one byte per instance that says whether the record was written. The render
// backward writes the records of the instances some warp of their tile kept (the others'
// gradients are exact zeros) and sets their bytes; the bytes start at zero (cleared
// before the render backward), so the preprocess backward reads only written records.
constexpr int kRecordFloat4 = 3;

struct ScratchLayout {
  size_t records, written, total;
  __host__ __device__ explicit ScratchLayout(int64_t cap) {
    const size_t c = (size_t)(cap > 0 ? cap : 1);
    records = 0;
    written = align256(sizeof(float) * 4 * kRecordFloat4 * c);
    total = align256(written + c);
  }
};

// ---------------------------------------------------------------------------
// Scalar math whose exact rounding sequence the CPU oracle reproduces.
// ---------------------------------------------------------------------------

// Bounded sense-reversing barrier across the blocks of a cooperative launch (every block
// resident). Lives in the image workspace's header, after CfgsCounts; `arrived` must be
// zero at launch. A block that waits longer than kGridBarrierMaxPolls polls raises
// CFGS_FLAG_BARRIER_TIMEOUT and gets false back; its kernel then returns, and the other
// blocks give up at their next wait the same way.
struct GridBarrier {
  unsigned int arrived, generation;
};
constexpr size_t kGridBarrierOffset = 128;  // bytes into the image workspace
static_assert(sizeof(CfgsCounts) <= kGridBarrierOffset && kGridBarrierOffset + sizeof(GridBarrier) <= 256,
              "the barrier follows the counts inside the 256-byte header");
constexpr uint32_t kGridBarrierMaxPolls = 1u << 22;

__device__ __forceinline__ bool grid_barrier(GridBarrier* b, uint32_t* flags) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &b->generation;
    const unsigned int g0 = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(&b->arrived, 1u) == gridDim.x - 1) {  // last to arrive releases the others
      atomicExch(&b->arrived, 0u);
      __threadfence();
      atomicAdd(&b->generation, 1u);
    } else {
      uint32_t polls = 0;
      while (*gen == g0) {
        if (++polls > kGridBarrierMaxPolls) {
          ok = 0;
          atomicOr(flags, CFGS_FLAG_BARRIER_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Sums six float64 values over the warp by a transposing reduction: each step halves the
// values a lane carries (4 + 2 + 1 shuffle-and-add steps, then two plain steps), 9 float64
// adds per lane instead of 30 for six butterflies. Lane 4k ends with the total of value k.
__device__ __forceinline__ double warp_sum6_f64(const double (&t)[6], int lane) {
  double v[8] = {t[0], t[1], t[2], t[3], t[4], t[5], 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const bool up = lane & 16;
    const double send = up ? v[k] : v[k + 4];
    const double keep = up ? v[k + 4] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool up = lane & 8;
    const double send = up ? v[k] : v[k + 2];
    const double keep = up ? v[k + 2] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  {
    const bool up = lane & 4;
    const double send = up ? v[0] : v[1];
    const double keep = up ? v[1] : v[0];
    v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
  return v[0];
}

// exp(x) in float: Cody–Waite reduction x = k ln2 + r (|r| <= ln2/2) with ln2 split
// into a 15-bit head (so k*head is exact) and a tail, then the degree-7 Taylor
// polynomial of e^r in Horner form (truncation error < 1e-8 relative), then an
// exact two-step scaling by 2^k. Every operation is an IEEE-rounded float op or an
// fma, so the same sequence in C gives the same bits.
__device__ __forceinline__ float exp_ref(float x) {
  if (x != x) return x;
  if (x < -104.0f) return 0.0f;
  if (x > 88.75f) return __int_as_float(0x7f800000);
  const float kLog2e = 1.4426950216293335f;
  const float kLn2Hi = 0.693145751953125f;
  const float kLn2Lo = 1.428606765330187e-06f;
  float kf = rintf(x * kLog2e);
  float r = fmaf(-kf, kLn2Hi, x);
  r = fmaf(-kf, kLn2Lo, r);
  float p = 0.00019841270113829523f;
  p = fmaf(p, r, 0.0013888889225199819f);
  p = fmaf(p, r, 0.008333333767950535f);
  p = fmaf(p, r, 0.0416666679084301f);
  p = fmaf(p, r, 0.1666666716337204f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int k = (int)kf;
  int k1 = k >> 1;
  int k2 = k - k1;
  float s1 = __int_as_float((k1 + 127) << 23);
  float s2 = __int_as_float((k2 + 127) << 23);
  return (p * s1) * s2;
}

// Exponent of the 2D Gaussian at pixel offset (dx, dy) = (mean - pixel), with the
// per-Gaussian factors pre-scaled as ca = -conic.a/2, cb = -conic.b, cc = -conic.c/2:
// power = ca dx^2 + cb dx dy + cc dy^2, evaluated in this exact order. Shared by the
// forward and backward render so the backward replays the forward's skip decisions.
__device__ __forceinline__ float gauss_power(float ca, float cb, float cc, float dx, float dy) {
  float e = cb * (dx * dy);
  e = fmaf(cc * dy, dy, e);
  return fmaf(ca * dx, dx, e);
}

// exp_ref for x in [-103, 0] (and NaN): the same operation sequence without the range
// guards, and the scaling by 2^k as one multiply — exact, and equal to exp_ref's
// two-step scaling, whenever the result is a normal float (k >= -125), which holds
// for every x the render kernels pass (see alpha_threshold).
__device__ __forceinline__ float exp_ref_inrange(float x) {
  const float kLog2e = 1.4426950216293335f;
  const float kLn2Hi = 0.693145751953125f;
  const float kLn2Lo = 1.428606765330187e-06f;
  float kf = rintf(x * kLog2e);
  float r = fmaf(-kf, kLn2Hi, x);
  r = fmaf(-kf, kLn2Lo, r);
  float p = 0.00019841270113829523f;
  p = fmaf(p, r, 0.0013888889225199819f);
  p = fmaf(p, r, 0.008333333767950535f);
  p = fmaf(p, r, 0.0416666679084301f);
  p = fmaf(p, r, 0.1666666716337204f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  return p * __int_as_float(((int)kf + 127) << 23);
}

// ---------------------------------------------------------------------------
// Packed FP32 pairs: one instruction performs two IEEE round-to-nearest operations
// (fma/mul/add .rn.f32x2), so each half is bit-identical to the scalar operation. The
// render kernels evaluate a lane's two pixels with them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)), "l"(f2_pack(c)));
  return f2_unpack(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(d);
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(d);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(d);
}
__device__ __forceinline__ float2 splat2(float a) { return make_float2(a, a); }

// gauss_power for the pixels (dx, dy.x) and (dx, dy.y): the same rounding sequence.
__device__ __forceinline__ float2 gauss_power2(float ca, float cb, float cc, float dx, float2 dy) {
  float2 e = mul2(splat2(cb), mul2(splat2(dx), dy));
  e = fma2(mul2(splat2(cc), dy), dy, e);
  const float cadx = ca * dx;
  return fma2(splat2(cadx), splat2(dx), e);
}

// exp_ref_inrange of both halves: the same rounding sequence (fmaf(-k, c, x) is
// fmaf(k, -c, x) exactly).
__device__ __forceinline__ float2 exp_ref_inrange2(float2 x) {
  const float2 t = mul2(x, splat2(1.4426950216293335f));
  const float2 kf = make_float2(rintf(t.x), rintf(t.y));
  float2 r = fma2(kf, splat2(-0.693145751953125f), x);
  r = fma2(kf, splat2(-1.428606765330187e-06f), r);
  float2 p = fma2(splat2(0.00019841270113829523f), r, splat2(0.0013888889225199819f));
  p = fma2(p, r, splat2(0.008333333767950535f));
  p = fma2(p, r, splat2(0.0416666679084301f));
  p = fma2(p, r, splat2(0.1666666716337204f));
  p = fma2(p, r, splat2(0.5f));
  p = fma2(p, r, splat2(1.0f));
  p = fma2(p, r, splat2(1.0f));
  const float2 sc = make_float2(__int_as_float(((int)kf.x + 127) << 23), __int_as_float(((int)kf.y + 127) << 23));
  return mul2(p, sc);
}

// ---------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async): the render kernels stage the next
// batch of instances while they composite the current one. The copying thread waits for
// its own copies (cp_async_wait_all) before a block barrier publishes them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ---------------------------------------------------------------------------
// mbarrier helpers for bulk and tensor copies into shared memory.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for phase `parity` of an mbarrier: at most max_polls try_wait polls; false
// if the phase did not complete (the caller raises an error flag and carries on).
constexpr uint32_t kMbarMaxPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t max_polls = kMbarMaxPolls) {
  for (uint32_t it = 0; it < max_polls; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Lower bound on the exponent of a Gaussian of opacity o that can still give
// alpha >= 1/255: below it, min(0.99, o exp_ref(power)) < 1/255 for certain, so the
// pixel can skip the exponential without changing any output. The bound sits 1e-3
// (in log space) under ln(1/(255 o)), far outside float error, and is clamped to
// -74 so the exponentials that do run stay in exp_ref_inrange's exact range; the
// clamp never hides a contribution for o <= 1e29.
__device__ __forceinline__ float alpha_threshold(float o) {
  float t = -logf(255.0f * o) - 1e-3f;
  return t != t ? -74.0f : fmaxf(t, -74.0f);
}

// Can any pixel of the box [x0, x1] x [y0, y1] get alpha >= 1/255 from the Gaussian
// centred at m with exponent power(d) = ca dx^2 + cb dx dy + cc dy^2 (d = m - pixel)?
// Maximises the concave exponent over the box (the centre if inside, otherwise the best
// point of each edge) and compares with the threshold tau with a 0.05 margin. Returns
// true (keep) whenever the quadratic is not negative definite.
__device__ __forceinline__ bool box_may_contribute(float2 m, float ca, float cb, float cc, float tau, float x0,
                                                   float x1, float y0, float y1) {
  if (!(ca < 0.0f && cc < 0.0f && 4.0f * ca * cc - cb * cb > 0.0f)) return true;
  const float dx0 = m.x - x1, dx1 = m.x - x0, dy0 = m.y - y1, dy1 = m.y - y0;
  if (dx0 <= 0.0f && dx1 >= 0.0f && dy0 <= 0.0f && dy1 >= 0.0f) return true;
  float best = -INFINITY;
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float X = e ? dx1 : dx0;  // edge dx = X: maximise over dy
    const float dy = fminf(fmaxf(-cb * X / (2.0f * cc), dy0), dy1);
    best = fmaxf(best, ca * X * X + cb * X * dy + cc * dy * dy);
    const float Y = e ? dy1 : dy0;  // edge dy = Y: maximise over dx
    const float dx = fminf(fmaxf(-cb * Y / (2.0f * ca), dx0), dx1);
    best = fmaxf(best, ca * dx * dx + cb * dx * Y + cc * Y * Y);
  }
  return best >= tau - 0.05f;
}

// Real spherical-harmonics constants of utils/sh_utils.py:16-40 (degrees 0..3).
#define CFGS_SH_C0 0.28209479177387814f
#define CFGS_SH_C1 0.4886025119029199f
#define CFGS_SH_C2_0 1.0925484305920792f
#define CFGS_SH_C2_1 (-1.0925484305920792f)
#define CFGS_SH_C2_2 0.31539156525252005f
#define CFGS_SH_C2_3 (-1.0925484305920792f)
#define CFGS_SH_C2_4 0.5462742152960396f
#define CFGS_SH_C3_0 (-0.5900435899266435f)
#define CFGS_SH_C3_1 2.890611442640554f
#define CFGS_SH_C3_2 (-0.4570457994644658f)
#define CFGS_SH_C3_3 0.3731763325901154f
#define CFGS_SH_C3_4 (-0.4570457994644658f)
#define CFGS_SH_C3_5 1.445305721320277f
#define CFGS_SH_C3_6 (-0.5900435899266435f)

// Alpha-compositing thresholds of the published 3DGS rasteriser.
#define CFGS_ALPHA_MAX 0.99f
#define CFGS_ALPHA_MIN 0.003921568859368563f  // 1/255 in float
#define CFGS_T_MIN 0.0001f
#define CFGS_NEAR_Z 0.2f

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

// Host-side launch check; returns CFGS_ERR_LAUNCH from the calling entry point.
#define CFGS_CHECK_LAUNCH(settings_debug, stream)                       \
  do {                                                                  \
    cudaError_t e_ = cudaGetLastError();                                \
    if (e_ != cudaSuccess) return CFGS_ERR_LAUNCH;                      \
    if (settings_debug) {                                               \
      e_ = cudaStreamSynchronize((cudaStream_t)(stream));               \
      if (e_ != cudaSuccess) return CFGS_ERR_LAUNCH;                    \
    }                                                                   \
  } while (0)

}  // namespace cfgs
