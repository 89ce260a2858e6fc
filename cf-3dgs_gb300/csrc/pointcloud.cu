// Local-Gaussian initialisation of a CF-3DGS frame (the steps before each pose solve,
// trainer/trainer.py:489-512 and scene/gaussian_model_cf.py:175-210):
//   - depth -> camera-space points: kornia depth_to_3d(normalize_points=False), i.e.
//     ((u - cx) / fx * d, (v - cy) / fy * d, d) at pixel (u, v);
//   - voxel down-sampling: Open3D voxel_down_sample — voxel index
//     floor((p - (min - s/2)) / s) in float64, each voxel's points and colours averaged
//     in float64 in input order; here the voxels come out sorted by their index;
//   - initial scales: simple-knn distCUDA2 — per point the mean squared distance to its
//     three nearest other points (missing neighbours count as FLT_MAX).
// kornia, Open3D and simple-knn are unpinned dependencies of the reference
// (requirements.txt; .gitmodules:1-3); their published algorithms are restated.
//
// kNN search: points sorted by 30-bit Morton code, cut into boxes of 32 consecutive
// points and super-boxes of 32 boxes, each with its bounding box. A point (one thread,
// in Morton order so a warp's points are neighbours) seeds its best three from its own
// box, then visits the super-boxes and boxes whose distance lower bound can still beat
// its third-best (with a 1e-5 relative margin against rounding) and checks their points.
// The result is the exact three smallest squared distances.
#include <cfloat>
#include <cmath>

#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

constexpr int kKnnBox = 32;
constexpr int kKnnSuper = 32;  // boxes per super-box
constexpr float kKnnMargin = 1.0f + 1e-5f;

// Squared distance with one fixed rounding sequence (the oracle performs the same).
__host__ __device__ __forceinline__ float dist2_ref(float ax, float ay, float az, float bx, float by, float bz) {
  const float dx = ax - bx, dy = ay - by, dz = az - bz;
  return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// ---- depth -> points ---------------------------------------------------------------
__global__ void __launch_bounds__(256) k_depth_to_points(int H, int W, const float* __restrict__ depth, float fx,
                                                         float fy, float cx, float cy, float* __restrict__ xyz) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)H * W) return;
  const int u = (int)(i % W), v = (int)(i / W);
  const float d = depth[i];
  xyz[3 * i + 0] = __fmul_rn(__fdiv_rn(__fsub_rn((float)u, cx), fx), d);
  xyz[3 * i + 1] = __fmul_rn(__fdiv_rn(__fsub_rn((float)v, cy), fy), d);
  xyz[3 * i + 2] = d;
}

// ---- bounds ---------------------------------------------------------------------------
// Per-axis min and max of n points into out[0..5] (min xyz, max xyz), one block.
__global__ void __launch_bounds__(1024) k_bounds(int64_t n, const float* __restrict__ xyz, float* __restrict__ out) {
  __shared__ float sh[6][32];
  float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float c = xyz[3 * i + a];
      v[a] = fminf(v[a], c);
      v[3 + a] = fmaxf(v[3 + a], c);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    float x = v[a];
    for (int o = 16; o > 0; o >>= 1) {
      const float y = __shfl_xor_sync(0xffffffffu, x, o);
      x = a < 3 ? fminf(x, y) : fmaxf(x, y);
    }
    if (lane == 0) sh[a][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int a = threadIdx.x;
    float x = sh[a][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) x = a < 3 ? fminf(x, sh[a][w]) : fmaxf(x, sh[a][w]);
    out[a] = x;
  }
}

// ---- voxel down-sampling -----------------------------------------------------------
struct VoxelGrid {
  double min_x, min_y, min_z, size;
  uint64_t ny, nz;  // voxels along y and z (key = (ix ny + iy) nz + iz)
};

__global__ void __launch_bounds__(256) k_voxel_keys(int64_t n, const float* __restrict__ xyz, VoxelGrid g,
                                                    uint32_t* __restrict__ key_lo, uint32_t* __restrict__ key_hi,
                                                    uint32_t* __restrict__ idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double rx = ((double)xyz[3 * i + 0] - g.min_x) / g.size;
  const double ry = ((double)xyz[3 * i + 1] - g.min_y) / g.size;
  const double rz = ((double)xyz[3 * i + 2] - g.min_z) / g.size;
  const uint64_t k = ((uint64_t)floor(rx) * g.ny + (uint64_t)floor(ry)) * g.nz + (uint64_t)floor(rz);
  key_lo[i] = (uint32_t)k;
  if (key_hi) key_hi[i] = (uint32_t)(k >> 32);
  if (idx) idx[i] = (uint32_t)i;
}

__global__ void __launch_bounds__(256) k_gather_u32(int64_t n, const uint32_t* __restrict__ src,
                                                    const uint32_t* __restrict__ idx, uint32_t* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

// heads[i] = 1 where a new voxel starts in the sorted order (keys compared in full).
__global__ void __launch_bounds__(256) k_voxel_heads(int64_t n, const uint32_t* __restrict__ lo,
                                                     const uint32_t* __restrict__ hi, uint32_t* __restrict__ heads) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool h = i == 0 || lo[i] != lo[i - 1];
  if (!h && hi) h = hi[i] != hi[i - 1];
  heads[i] = h ? 1u : 0u;
}

// Exclusive scan of heads into starts (one block; n fits in memory, voxel counts are
// modest) and the voxel count into *count: starts[v] = first sorted position of voxel v.
__global__ void __launch_bounds__(1024) k_voxel_starts(int64_t n, const uint32_t* __restrict__ heads,
                                                       uint32_t* __restrict__ starts, uint32_t* __restrict__ count) {
  __shared__ uint32_t sh[64];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  uint32_t carry = 0;
  for (int64_t base = 0; base < n; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const uint32_t h = i < n ? heads[i] : 0u;
    uint32_t x = h;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = lane < nw ? sh[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      sh[32 + lane] = w;
    }
    __syncthreads();
    const uint32_t incl = carry + x + (warp > 0 ? sh[32 + warp - 1] : 0u);
    if (h) starts[incl - 1] = (uint32_t)i;
    carry += sh[32 + nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    starts[carry] = (uint32_t)n;
    *count = carry;
  }
}

// One thread per voxel: float64 sums of its points and colours in input order (the
// sort is stable), averaged and rounded to float.
__global__ void __launch_bounds__(256) k_voxel_average(const uint32_t* __restrict__ count,
                                                       const uint32_t* __restrict__ starts,
                                                       const uint32_t* __restrict__ order,
                                                       const float* __restrict__ xyz, const float* __restrict__ rgb,
                                                       float* __restrict__ out_xyz, float* __restrict__ out_rgb) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= *count) return;
  const uint32_t b = starts[v], e = starts[v + 1];
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (uint32_t k = b; k < e; ++k) {
    const uint32_t i = order[k];
#pragma unroll
    for (int a = 0; a < 3; ++a) s[a] += (double)xyz[3 * (size_t)i + a];
    if (rgb) {
#pragma unroll
      for (int a = 0; a < 3; ++a) s[3 + a] += (double)rgb[3 * (size_t)i + a];
    }
  }
  const double inv = (double)(e - b);
#pragma unroll
  for (int a = 0; a < 3; ++a) out_xyz[3 * (size_t)v + a] = (float)(s[a] / inv);
  if (rgb && out_rgb) {
#pragma unroll
    for (int a = 0; a < 3; ++a) out_rgb[3 * (size_t)v + a] = (float)(s[3 + a] / inv);
  }
}

// ---- kNN -------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void __launch_bounds__(256) k_morton(int64_t n, const float* __restrict__ xyz,
                                                const float* __restrict__ bounds, uint32_t* __restrict__ code,
                                                uint32_t* __restrict__ idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float lo = bounds[a], ext = bounds[3 + a] - lo;
    const float t = ext > 0.f ? (xyz[3 * i + a] - lo) / ext : 0.f;
    q[a] = (uint32_t)fminf(fmaxf(t * 1024.f, 0.f), 1023.f);
  }
  code[i] = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
  idx[i] = (uint32_t)i;
}

// Sorted points as float4 (x, y, z, original index bits).
__global__ void __launch_bounds__(256) k_gather_points(int64_t n, const float* __restrict__ xyz,
                                                       const uint32_t* __restrict__ order, float4* __restrict__ pts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t j = order[i];
  pts[i] = make_float4(xyz[3 * (size_t)j], xyz[3 * (size_t)j + 1], xyz[3 * (size_t)j + 2], __uint_as_float(j));
}

// Bounding boxes of consecutive groups of `group` items: from points (boxes) or from
// finer boxes (super-boxes). Box b = (min.xyz, max.xyz) in two float4.
__global__ void __launch_bounds__(256) k_boxes_from_points(int64_t n, const float4* __restrict__ pts,
                                                           float4* __restrict__ box) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t s = b * kKnnBox;
  if (s >= n) return;
  float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
  for (int64_t i = s; i < min(n, s + kKnnBox); ++i) {
    const float4 p = pts[i];
    lo.x = fminf(lo.x, p.x); lo.y = fminf(lo.y, p.y); lo.z = fminf(lo.z, p.z);
    hi.x = fmaxf(hi.x, p.x); hi.y = fmaxf(hi.y, p.y); hi.z = fmaxf(hi.z, p.z);
  }
  box[2 * b] = lo;
  box[2 * b + 1] = hi;
}

__global__ void __launch_bounds__(256) k_boxes_from_boxes(int64_t nbox, const float4* __restrict__ box,
                                                          float4* __restrict__ sup) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t s = b * kKnnSuper;
  if (s >= nbox) return;
  float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
  for (int64_t i = s; i < min(nbox, s + kKnnSuper); ++i) {
    const float4 l = box[2 * i], h = box[2 * i + 1];
    lo.x = fminf(lo.x, l.x); lo.y = fminf(lo.y, l.y); lo.z = fminf(lo.z, l.z);
    hi.x = fmaxf(hi.x, h.x); hi.y = fmaxf(hi.y, h.y); hi.z = fmaxf(hi.z, h.z);
  }
  sup[2 * b] = lo;
  sup[2 * b + 1] = hi;
}

// Squared distance from q to the box (0 inside), a lower bound of every member's.
__device__ __forceinline__ float box_dist2(const float4& q, const float4& lo, const float4& hi) {
  const float gx = fmaxf(fmaxf(lo.x - q.x, q.x - hi.x), 0.f);
  const float gy = fmaxf(fmaxf(lo.y - q.y, q.y - hi.y), 0.f);
  const float gz = fmaxf(fmaxf(lo.z - q.z, q.z - hi.z), 0.f);
  return fmaf(gz, gz, fmaf(gy, gy, gx * gx));
}

__device__ __forceinline__ void best3_insert(float (&b)[3], float d) {
  if (d < b[2]) {
    if (d < b[1]) {
      b[2] = b[1];
      if (d < b[0]) {
        b[1] = b[0];
        b[0] = d;
      } else {
        b[1] = d;
      }
    } else {
      b[2] = d;
    }
  }
}

__device__ __forceinline__ void scan_box(const float4& q, uint32_t self, const float4* __restrict__ pts, int64_t n,
                                         int64_t box, float (&b)[3]) {
  const int64_t s = box * kKnnBox, e = min(n, s + kKnnBox);
  for (int64_t i = s; i < e; ++i) {
    const float4 p = pts[i];
    if (__float_as_uint(p.w) == self) continue;
    best3_insert(b, dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z));
  }
}

__global__ void __launch_bounds__(256) k_knn3(int64_t n, const float4* __restrict__ pts,
                                              const float4* __restrict__ box, const float4* __restrict__ sup,
                                              float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 q = pts[i];
  const uint32_t self = __float_as_uint(q.w);
  const int64_t nbox = (n + kKnnBox - 1) / kKnnBox;
  const int64_t nsup = (nbox + kKnnSuper - 1) / kKnnSuper;
  float b[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  const int64_t own = i / kKnnBox;
  scan_box(q, self, pts, n, own, b);
  for (int64_t sb = 0; sb < nsup; ++sb) {
    if (box_dist2(q, sup[2 * sb], sup[2 * sb + 1]) > b[2] * kKnnMargin) continue;
    const int64_t e = min(nbox, (sb + 1) * kKnnSuper);
    for (int64_t bx = sb * kKnnSuper; bx < e; ++bx) {
      if (bx == own) continue;
      if (box_dist2(q, box[2 * bx], box[2 * bx + 1]) > b[2] * kKnnMargin) continue;
      scan_box(q, self, pts, n, bx, b);
    }
  }
  out[self] = ((b[0] + b[1]) + b[2]) / 3.0f;
}

// ---- workspaces ----------------------------------------------------------------------
struct PcLayout {
  size_t keys, vals, extra, extra2, bounds, counts, totals, pts, box, sup, total;
  explicit PcLayout(int64_t n) {
    const size_t c = pingpong_stride(n);
    const int64_t nbox = (n + kKnnBox - 1) / kKnnBox;
    const int64_t nsup = (nbox + kKnnSuper - 1) / kKnnSuper;
    size_t o = 0;
    keys = o;   o = align256(o + sizeof(uint32_t) * 2 * c);
    vals = o;   o = align256(o + sizeof(uint32_t) * 2 * c);
    extra = o;  o = align256(o + sizeof(uint32_t) * (c + 1));
    extra2 = o; o = align256(o + sizeof(uint32_t) * (c + 1));
    bounds = o; o = align256(o + sizeof(float) * 8);
    counts = o; o = align256(o + sizeof(uint32_t) * kSortDigits * (size_t)sort_chunks(n, kTileChunk));
    totals = o; o = align256(o + sizeof(uint32_t) * kSortDigits * kMaxTilePasses);
    pts = o;    o = align256(o + sizeof(float4) * (size_t)(n > 0 ? n : 1));
    box = o;    o = align256(o + 2 * sizeof(float4) * (size_t)(nbox > 0 ? nbox : 1));
    sup = o;    o = align256(o + 2 * sizeof(float4) * (size_t)(nsup > 0 ? nsup : 1));
    total = o;
  }
};

}  // namespace cfgs

using namespace cfgs;

extern "C" int cfgs_depth_to_points(int32_t height, int32_t width, const float* depth, float fx, float fy, float cx,
                                    float cy, float* xyz, void* stream) {
  if (height <= 0 || width <= 0 || !depth || !xyz || (int64_t)height * width > 0x7fffffffll)
    return CFGS_ERR_INVALID_ARGUMENT;
  const int64_t n = (int64_t)height * width;
  k_depth_to_points<<<div_up(n, 256), 256, 0, (cudaStream_t)stream>>>(height, width, depth, fx, fy, cx, cy, xyz);
  CFGS_CHECK_LAUNCH(0, stream);
  return CFGS_OK;
}

extern "C" size_t cfgs_pointcloud_workspace_bytes(int64_t num_points) {
  return num_points < 0 || num_points > 0x7fffffffll ? 0 : PcLayout(num_points).total;
}

extern "C" int cfgs_knn3_mean_dist2(int64_t num_points, const float* xyz, void* workspace, float* dist2,
                                    void* stream) {
  if (num_points < 0 || num_points > 0x7fffffffll || (num_points > 0 && (!xyz || !workspace || !dist2)))
    return CFGS_ERR_INVALID_ARGUMENT;
  const int64_t n = num_points;
  if (n == 0) return CFGS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  PcLayout L(n);
  char* w = static_cast<char*>(workspace);
  const size_t c = pingpong_stride(n);
  uint32_t* keys[2] = {reinterpret_cast<uint32_t*>(w + L.keys), reinterpret_cast<uint32_t*>(w + L.keys) + c};
  uint32_t* vals[2] = {reinterpret_cast<uint32_t*>(w + L.vals), reinterpret_cast<uint32_t*>(w + L.vals) + c};
  float* bounds = reinterpret_cast<float*>(w + L.bounds);
  float4* pts = reinterpret_cast<float4*>(w + L.pts);
  float4* box = reinterpret_cast<float4*>(w + L.box);
  float4* sup = reinterpret_cast<float4*>(w + L.sup);
  k_bounds<<<1, 1024, 0, st>>>(n, xyz, bounds);
  k_morton<<<div_up(n, 256), 256, 0, st>>>(n, xyz, bounds, keys[0], vals[0]);
  int res = 0;
  int s = sort_pairs(keys, vals, n, 30, reinterpret_cast<uint32_t*>(w + L.counts),
                     reinterpret_cast<uint32_t*>(w + L.totals), st, &res);
  if (s != CFGS_OK) return s;
  k_gather_points<<<div_up(n, 256), 256, 0, st>>>(n, xyz, vals[res], pts);
  const int64_t nbox = (n + kKnnBox - 1) / kKnnBox;
  const int64_t nsup = (nbox + kKnnSuper - 1) / kKnnSuper;
  k_boxes_from_points<<<div_up(nbox, 256), 256, 0, st>>>(n, pts, box);
  k_boxes_from_boxes<<<div_up(nsup, 256), 256, 0, st>>>(nbox, box, sup);
  k_knn3<<<div_up(n, 256), 256, 0, st>>>(n, pts, box, sup, dist2);
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}

extern "C" int cfgs_voxel_down_sample(int64_t num_points, const float* xyz, const float* rgb, double voxel_size,
                                      void* workspace, float* out_xyz, float* out_rgb, int64_t* num_voxels,
                                      void* stream) {
  if (num_points < 0 || num_points > 0x7fffffffll || !num_voxels || !(voxel_size > 0.0))
    return CFGS_ERR_INVALID_ARGUMENT;
  if (num_points > 0 && (!xyz || !workspace || !out_xyz || (rgb && !out_rgb))) return CFGS_ERR_INVALID_ARGUMENT;
  *num_voxels = 0;
  const int64_t n = num_points;
  if (n == 0) return CFGS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  PcLayout L(n);
  char* w = static_cast<char*>(workspace);
  const size_t c = pingpong_stride(n);
  uint32_t* keys[2] = {reinterpret_cast<uint32_t*>(w + L.keys), reinterpret_cast<uint32_t*>(w + L.keys) + c};
  uint32_t* vals[2] = {reinterpret_cast<uint32_t*>(w + L.vals), reinterpret_cast<uint32_t*>(w + L.vals) + c};
  uint32_t* extra = reinterpret_cast<uint32_t*>(w + L.extra);
  float* bounds = reinterpret_cast<float*>(w + L.bounds);
  uint32_t* counts = reinterpret_cast<uint32_t*>(w + L.counts);
  uint32_t* totals = reinterpret_cast<uint32_t*>(w + L.totals);
  k_bounds<<<1, 1024, 0, st>>>(n, xyz, bounds);
  float hb[6];
  if (cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  // Open3D: min bound - s/2; the span must index with int
  VoxelGrid g;
  g.size = voxel_size;
  g.min_x = (double)hb[0] - 0.5 * voxel_size;
  g.min_y = (double)hb[1] - 0.5 * voxel_size;
  g.min_z = (double)hb[2] - 0.5 * voxel_size;
  uint64_t dim[3];
  const double lo[3] = {g.min_x, g.min_y, g.min_z};
  for (int a = 0; a < 3; ++a) {
    const double span = ((double)hb[3 + a] + 0.5 * voxel_size - lo[a]) / voxel_size;
    if (!(span < 2147483647.0)) return CFGS_ERR_TOO_LARGE;
    dim[a] = (uint64_t)std::floor(((double)hb[3 + a] - lo[a]) / voxel_size) + 1;
  }
  g.ny = dim[1];
  g.nz = dim[2];
  const double cells = (double)dim[0] * (double)dim[1] * (double)dim[2];
  if (cells >= 18446744073709551615.0) return CFGS_ERR_TOO_LARGE;
  const bool wide = cells > 4294967295.0;
  // keys[0] = low 32 key bits, extra = high 32 bits (wide grids), vals[0] = input index.
  // Wide keys sort as two stable LSD groups: low halves, then high halves.
  uint32_t* extra2 = reinterpret_cast<uint32_t*>(w + L.extra2);
  k_voxel_keys<<<div_up(n, 256), 256, 0, st>>>(n, xyz, g, keys[0], wide ? extra : nullptr, vals[0]);
  int r1 = 0;
  int s = sort_pairs(keys, vals, n, 32, counts, totals, st, &r1);
  if (s != CFGS_OK) return s;
  uint32_t *lo_sorted = keys[r1], *hi_sorted = nullptr, *order = vals[r1], *free_buf = vals[r1 ^ 1];
  if (wide) {
    uint32_t* k2[2] = {keys[r1 ^ 1], keys[r1]};
    uint32_t* v2[2] = {vals[r1], vals[r1 ^ 1]};
    k_gather_u32<<<div_up(n, 256), 256, 0, st>>>(n, extra, vals[r1], k2[0]);  // high halves, round-1 order
    int r2 = 0;
    s = sort_pairs(k2, v2, n, 32, counts, totals, st, &r2);
    if (s != CFGS_OK) return s;
    hi_sorted = k2[r2];
    order = v2[r2];
    free_buf = v2[r2 ^ 1];
    k_voxel_keys<<<div_up(n, 256), 256, 0, st>>>(n, xyz, g, extra, nullptr, nullptr);  // low halves by input
    lo_sorted = k2[r2 ^ 1];
    k_gather_u32<<<div_up(n, 256), 256, 0, st>>>(n, extra, order, lo_sorted);
  }
  uint32_t* heads = free_buf;
  k_voxel_heads<<<div_up(n, 256), 256, 0, st>>>(n, lo_sorted, hi_sorted, heads);
  uint32_t* starts = extra2;  // n + 1 entries
  uint32_t* dcount = reinterpret_cast<uint32_t*>(bounds + 6);
  k_voxel_starts<<<1, 1024, 0, st>>>(n, heads, starts, dcount);
  k_voxel_average<<<div_up(n, 256), 256, 0, st>>>(dcount, starts, order, xyz, rgb, out_xyz, out_rgb);
  uint32_t hc = 0;
  if (cudaMemcpyAsync(&hc, dcount, sizeof(hc), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  *num_voxels = hc;
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}
