// Optimisation of the Gaussian parameters (CF-3DGS global refinement and local fitting,
// trainer/cf3dgs_trainer.py:144-170 / 232-259): the Adam step over every parameter
// group, the densification statistics and densify-and-prune of
// scene/gaussian_model_cf.py:242-301 and 605-719, on device-resident arrays.
//
// Adam: one launch for all groups (xyz, f_dc, f_rest, opacity, scaling, rotation) with
// the operation sequence of torch's multi-tensor Adam (non-capturable):
//   m = lerp(m, g, 1 - b1) = fma(1 - b1, g - m, m); v = fma(1 - b2, g * g, v * b2);
//   p = fma(-lr / bc1, m / (sqrt(v) / sqrt(bc2) + eps), p)
// with the per-group scalars formed on the host as torch forms them.
//
// Densify and prune (densify_and_prune with grads = accum / denom, nan -> 0):
//   clone  = |grad| >= max_grad and max(exp(scaling)) <= percent_dense * extent
//   split  = |grad| >= max_grad and max(exp(scaling)) >  percent_dense * extent
//   prune  = sigmoid(opacity) < min_opacity, or (with the screen test enabled)
//            max(exp(scaling)) > 0.1 * extent (the screen-size term is always false
//            then: densification resets max_radii2D to zero)
// The result lists, in this order: the originals that are neither split nor pruned;
// the clones (copies of the raw parameters) whose source is not pruned; then two blocks
// of split children (copy 0 of every split point, then copy 1) not pruned, each child
// at xyz + R(q) (exp(scaling) * z), scaling log(exp(scaling) / 1.6), the rest copied.
// z are the caller's standard-normal draws, [2, splits, 3]. New rows get zero Adam
// moments; the statistics restart at zero.
#include <cmath>

#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

constexpr int kMaxAdamGroups = 8;

struct AdamGroups {
  float* p[kMaxAdamGroups];
  const float* g[kMaxAdamGroups];
  float* m[kMaxAdamGroups];
  float* v[kMaxAdamGroups];
  int64_t begin[kMaxAdamGroups + 1];  // flattened ranges of 4-element items
  int64_t numel[kMaxAdamGroups];
  float step_size[kMaxAdamGroups];    // -lr / bc1
  float bc2_sqrt[kMaxAdamGroups];
  float eps[kMaxAdamGroups];
  float w1, b2, w2;
  int count;
};

__device__ __forceinline__ void adam_elem(const AdamGroups& a, int k, float g, float& m, float& v, float& p) {
  m = fmaf(a.w1, g - m, m);
  v = v * a.b2;
  v = fmaf(a.w2, g * g, v);
  float denom = sqrtf(v) / a.bc2_sqrt[k];
  denom = denom + a.eps[k];
  p = fmaf(a.step_size[k], m / denom, p);
}

// One thread per 4 consecutive elements of a group (begin[] counts 4-element items, each
// group padded to a whole item): vector loads and stores where the item is whole and the
// arrays 16-byte aligned, scalar ones otherwise.
__global__ void __launch_bounds__(256) k_gaussian_adam(AdamGroups a) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.begin[a.count]) return;
  int k = 0;
  while (k + 1 < a.count && t >= a.begin[k + 1]) ++k;
  const int64_t e0 = 4 * (t - a.begin[k]);
  const int64_t numel = a.numel[k];
  float* P = a.p[k];
  const float* G = a.g[k];
  float* Mv = a.m[k];
  float* Vv = a.v[k];
  const bool vec = e0 + 3 < numel && ((((uintptr_t)P) | ((uintptr_t)G) | ((uintptr_t)Mv) | ((uintptr_t)Vv)) & 15) == 0;
  if (vec) {
    const float4 g4 = *reinterpret_cast<const float4*>(G + e0);
    float4 m4 = *reinterpret_cast<float4*>(Mv + e0), v4 = *reinterpret_cast<float4*>(Vv + e0);
    float4 p4 = *reinterpret_cast<float4*>(P + e0);
    adam_elem(a, k, g4.x, m4.x, v4.x, p4.x);
    adam_elem(a, k, g4.y, m4.y, v4.y, p4.y);
    adam_elem(a, k, g4.z, m4.z, v4.z, p4.z);
    adam_elem(a, k, g4.w, m4.w, v4.w, p4.w);
    *reinterpret_cast<float4*>(Mv + e0) = m4;
    *reinterpret_cast<float4*>(Vv + e0) = v4;
    *reinterpret_cast<float4*>(P + e0) = p4;
  } else {
    for (int64_t e = e0; e < min(numel, e0 + 4); ++e) {
      float m = Mv[e], v = Vv[e], p = P[e];
      adam_elem(a, k, G[e], m, v, p);
      Mv[e] = m;
      Vv[e] = v;
      P[e] = p;
    }
  }
}

// xyz_gradient_accum[i] += |grad2D[i, :2]|, denom[i] += 1 where radii[i] > 0
// (add_densification_stats with the visibility filter).
__global__ void __launch_bounds__(256) k_densify_stats(int64_t n, const int32_t* __restrict__ radii,
                                                       const float* __restrict__ grad2D, float* __restrict__ accum,
                                                       float* __restrict__ denom) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || radii[i] <= 0) return;
  const float gx = grad2D[3 * i], gy = grad2D[3 * i + 1];
  accum[i] += sqrtf(gx * gx + gy * gy);
  denom[i] += 1.0f;
}

struct DensifyParams {
  float max_grad, min_opacity, extent, percent_dense;
  int prune_big;
};

__device__ __forceinline__ float max_scale(const float* s) { return fmaxf(fmaxf(expf(s[0]), expf(s[1])), expf(s[2])); }

// Per point: bit 0 keep original, bit 1 kept clone, bit 2 split, bit 3 kept children.
__global__ void __launch_bounds__(256) k_densify_classify(int64_t n, const float* __restrict__ accum,
                                                          const float* __restrict__ denom,
                                                          const float* __restrict__ scaling,
                                                          const float* __restrict__ opacity, DensifyParams d,
                                                          uint32_t* __restrict__ cls) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float g = accum[i] / denom[i];
  if (g != g) g = 0.0f;
  const float smax = max_scale(scaling + 3 * i);
  const float thr = d.percent_dense * d.extent;
  const bool hot = fabsf(g) >= d.max_grad;
  const bool clone = hot && smax <= thr;
  const bool split = hot && smax > thr;
  const float op = 1.0f / (1.0f + expf(-opacity[i]));
  const bool low = op < d.min_opacity;
  const bool big = d.prune_big && smax > 0.1f * d.extent;
  // children: scaling log(exp(s) / 1.6) per axis
  float cs[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) cs[a] = logf(expf(scaling[3 * i + a]) / 1.6f);
  const bool child_big = d.prune_big && max_scale(cs) > 0.1f * d.extent;
  uint32_t c = 0;
  if (!split && !(low || big)) c |= 1u;
  if (clone && !(low || big)) c |= 2u;
  if (split) c |= 4u;
  if (split && !(low || child_big)) c |= 8u;
  cls[i] = c;
}

// Exclusive scans of the four class bits over the points, in three launches: per-block
// counts (1024 points per block), a scan of the block counts (one block; totals in
// tot[4]), then each block's exclusive scan offset by its block prefix.
constexpr int kDensScanBlock = 1024;

__device__ __forceinline__ void block_scan4(uint32_t c, uint32_t (*sh)[32], uint32_t (&excl)[4], uint32_t (&all)[4]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  uint32_t x[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const uint32_t f = (c >> b) & 1u;
    uint32_t s = f;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane == 31) sh[b][warp] = s;
    x[b] = s - f;
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    uint32_t before = 0, total = 0;
    for (int w = 0; w < nw; ++w) {
      const uint32_t t = sh[b][w];
      if (w < warp) before += t;
      total += t;
    }
    excl[b] = before + x[b];
    all[b] = total;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kDensScanBlock) k_densify_block_counts(int64_t n, const uint32_t* __restrict__ cls,
                                                                       uint32_t* __restrict__ bcount) {
  __shared__ uint32_t sh[4][32];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t excl[4], all[4];
  block_scan4(i < n ? cls[i] : 0u, sh, excl, all);
  if (threadIdx.x < 4) bcount[4 * (size_t)blockIdx.x + threadIdx.x] = all[threadIdx.x];
}

__global__ void __launch_bounds__(1024) k_densify_block_prefix(int nblocks, uint32_t* __restrict__ bcount,
                                                               uint32_t* __restrict__ tot) {
  __shared__ uint32_t sh[4 * 32];  // per warp (32) and column (4)
  const int b = threadIdx.x & 3;  // four columns, 256 threads each
  const int lane = threadIdx.x & 31;
  // column b, strided by 4: thread handles blocks j = (threadIdx.x >> 2) + 256 k
  uint32_t carry = 0;
  for (int base = 0; base < nblocks; base += 256) {
    const int j = base + (threadIdx.x >> 2);
    const uint32_t v = j < nblocks ? bcount[4 * (size_t)j + b] : 0u;
    // inclusive scan over j within the column: lanes of a warp hold 8 consecutive j of
    // each of the 4 columns (lane = 4 * jj + b)
    uint32_t x = v;
    for (int o = 4; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const int warp = threadIdx.x >> 5;
    if (lane >= 28) sh[4 * warp + (lane - 28)] = x;  // warp totals per column
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < 32; ++w) {
      const uint32_t t = sh[4 * w + b];
      if (w < warp) before += t;
      total += t;
    }
    if (j < nblocks) bcount[4 * (size_t)j + b] = carry + before + x - v;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x < 4) tot[b] = carry;
}

__global__ void __launch_bounds__(kDensScanBlock) k_densify_positions(int64_t n, const uint32_t* __restrict__ cls,
                                                                    const uint32_t* __restrict__ bprefix,
                                                                    uint32_t* __restrict__ pos) {
  __shared__ uint32_t sh[4][32];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t excl[4], all[4];
  block_scan4(i < n ? cls[i] : 0u, sh, excl, all);
  if (i < n) {
#pragma unroll
    for (int b = 0; b < 4; ++b) pos[4 * i + b] = bprefix[4 * (size_t)blockIdx.x + b] + excl[b];
  }
}

// out_src[r] = source point of output row r, out_kind[r] = 0 original, 1 clone,
// 2 + c child of copy c (and split_rank[r] = the point's index among the split points).
__global__ void __launch_bounds__(256) k_densify_map(int64_t n, const uint32_t* __restrict__ cls,
                                                     const uint32_t* __restrict__ pos,
                                                     const uint32_t* __restrict__ tot, uint32_t* __restrict__ out_src,
                                                     uint8_t* __restrict__ out_kind,
                                                     uint32_t* __restrict__ out_split_rank) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = cls[i];
  const uint32_t n_keep = tot[0], n_clone = tot[1], n_child = tot[3];
  if (c & 1u) {
    out_src[pos[4 * i]] = (uint32_t)i;
    out_kind[pos[4 * i]] = 0;
  }
  if (c & 2u) {
    const uint32_t r = n_keep + pos[4 * i + 1];
    out_src[r] = (uint32_t)i;
    out_kind[r] = 1;
  }
  if (c & 8u) {
#pragma unroll
    for (int cp = 0; cp < 2; ++cp) {
      const uint32_t r = n_keep + n_clone + cp * n_child + pos[4 * i + 3];
      out_src[r] = (uint32_t)i;
      out_kind[r] = (uint8_t)(2 + cp);
      out_split_rank[r] = pos[4 * i + 2];
    }
  }
}

// One parameter array (rows of `width` floats): out[r] = in[src[r]] (zero for new rows
// when zero_new, i.e. Adam moments); the child rows of xyz and scaling are special.
__global__ void __launch_bounds__(256) k_densify_gather(int64_t rows, int width, const float* __restrict__ in,
                                                        float* __restrict__ out, const uint32_t* __restrict__ src,
                                                        const uint8_t* __restrict__ kind, int zero_new) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * width) return;
  const int64_t r = t / width;
  const int c = (int)(t - r * width);
  out[t] = (zero_new && kind[r] != 0) ? 0.0f : in[(size_t)src[r] * width + c];
}

// Child rows (kind >= 2) of xyz (want_scaling = 0): xyz + R(normalize(q)) (exp(s) * z),
// or of scaling (want_scaling = 1): log(exp(s) / 1.6). R as build_rotation
// (utils/general_utils.py:76-97).
__global__ void __launch_bounds__(256) k_densify_children(int64_t rows, const uint32_t* __restrict__ src,
                                                          const uint8_t* __restrict__ kind,
                                                          const uint32_t* __restrict__ split_rank,
                                                          uint32_t num_split, const float* __restrict__ xyz,
                                                          const float* __restrict__ scaling,
                                                          const float* __restrict__ rotation,
                                                          const float* __restrict__ z, float* __restrict__ out,
                                                          int want_scaling) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows || kind[r] < 2) return;
  const uint32_t i = src[r];
  const int cp = kind[r] - 2;
  const float* q = rotation + 4 * (size_t)i;
  const float nrm = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const float qr = q[0] / nrm, qx = q[1] / nrm, qy = q[2] / nrm, qz = q[3] / nrm;
  const float R[9] = {1.f - 2.f * (qy * qy + qz * qz), 2.f * (qx * qy - qr * qz), 2.f * (qx * qz + qr * qy),
                      2.f * (qx * qy + qr * qz), 1.f - 2.f * (qx * qx + qz * qz), 2.f * (qy * qz - qr * qx),
                      2.f * (qx * qz - qr * qy), 2.f * (qy * qz + qr * qx), 1.f - 2.f * (qx * qx + qy * qy)};
  const float* zz = z + 3 * ((size_t)cp * num_split + split_rank[r]);
  float smp[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) smp[a] = expf(scaling[3 * (size_t)i + a]) * zz[a];
#pragma unroll
  for (int a = 0; a < 3; ++a)
    out[3 * r + a] = want_scaling ? logf(expf(scaling[3 * (size_t)i + a]) / 1.6f)
                                  : (R[3 * a] * smp[0] + R[3 * a + 1] * smp[1] + R[3 * a + 2] * smp[2]) +
                                        xyz[3 * (size_t)i + a];
}

}  // namespace cfgs

using namespace cfgs;

extern "C" int cfgs_gaussian_adam(int32_t num_groups, float* const* params, const float* const* grads,
                                  float* const* exp_avg, float* const* exp_avg_sq, const int64_t* numel,
                                  const double* lr, double beta1, double beta2, double eps, int64_t step,
                                  void* stream) {
  if (num_groups <= 0 || num_groups > kMaxAdamGroups || !params || !grads || !exp_avg || !exp_avg_sq || !numel ||
      !lr || step < 1)
    return CFGS_ERR_INVALID_ARGUMENT;
  AdamGroups a{};
  a.count = num_groups;
  // torch multi-tensor Adam: Python-float bias corrections, float32 operands
  const double bc1 = 1.0 - std::pow(beta1, (double)step);
  const double bc2 = 1.0 - std::pow(beta2, (double)step);
  a.w1 = (float)(1.0 - beta1);
  a.b2 = (float)beta2;
  a.w2 = (float)(1.0 - beta2);
  int64_t off = 0;
  for (int k = 0; k < num_groups; ++k) {
    if (numel[k] < 0 || (numel[k] > 0 && (!params[k] || !grads[k] || !exp_avg[k] || !exp_avg_sq[k])))
      return CFGS_ERR_INVALID_ARGUMENT;
    a.p[k] = params[k];
    a.g[k] = grads[k];
    a.m[k] = exp_avg[k];
    a.v[k] = exp_avg_sq[k];
    a.begin[k] = off;
    a.numel[k] = numel[k];
    off += (numel[k] + 3) / 4;
    a.step_size[k] = (float)(-(lr[k] / bc1));
    a.bc2_sqrt[k] = (float)std::sqrt(bc2);
    a.eps[k] = (float)eps;
  }
  a.begin[num_groups] = off;
  if (off == 0) return CFGS_OK;
  k_gaussian_adam<<<div_up(off, 256), 256, 0, (cudaStream_t)stream>>>(a);
  CFGS_CHECK_LAUNCH(0, stream);
  return CFGS_OK;
}

extern "C" int cfgs_densify_stats(int64_t num_gaussians, const int32_t* radii, const float* grad_means2D,
                                  float* grad_accum, float* denom, void* stream) {
  if (num_gaussians < 0 || (num_gaussians > 0 && (!radii || !grad_means2D || !grad_accum || !denom)))
    return CFGS_ERR_INVALID_ARGUMENT;
  if (num_gaussians == 0) return CFGS_OK;
  k_densify_stats<<<div_up(num_gaussians, 256), 256, 0, (cudaStream_t)stream>>>(num_gaussians, radii, grad_means2D,
                                                                                 grad_accum, denom);
  CFGS_CHECK_LAUNCH(0, stream);
  return CFGS_OK;
}

extern "C" size_t cfgs_densify_workspace_bytes(int64_t num_gaussians) {
  if (num_gaussians < 0) return 0;
  const size_t n = (size_t)(num_gaussians > 0 ? num_gaussians : 1);
  const size_t nb = (n + kDensScanBlock - 1) / kDensScanBlock;
  return align256(sizeof(uint32_t) * n) + align256(sizeof(uint32_t) * 4 * n) + align256(sizeof(uint32_t) * 4) +
         align256(sizeof(uint32_t) * 3 * n) + align256(sizeof(uint32_t) * 3 * n) + align256(3 * n) +
         align256(sizeof(uint32_t) * 4 * nb);
}

extern "C" int cfgs_densify_plan(int64_t num_gaussians, const float* grad_accum, const float* denom,
                                 const float* scaling, const float* opacity, float max_grad, float min_opacity,
                                 float extent, float percent_dense, int32_t prune_big, void* workspace,
                                 int64_t counts[4], void* stream) {
  if (num_gaussians < 0 || num_gaussians > 0x3fffffffll || !workspace || !counts) return CFGS_ERR_INVALID_ARGUMENT;
  if (num_gaussians > 0 && (!grad_accum || !denom || !scaling || !opacity)) return CFGS_ERR_INVALID_ARGUMENT;
  for (int b = 0; b < 4; ++b) counts[b] = 0;
  if (num_gaussians == 0) return CFGS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = num_gaussians;
  char* w = static_cast<char*>(workspace);
  uint32_t* cls = reinterpret_cast<uint32_t*>(w);
  uint32_t* pos = reinterpret_cast<uint32_t*>(w + align256(sizeof(uint32_t) * n));
  uint32_t* tot = reinterpret_cast<uint32_t*>(w + align256(sizeof(uint32_t) * n) + align256(sizeof(uint32_t) * 4 * n));
  const size_t o_src = align256(sizeof(uint32_t) * n) + align256(sizeof(uint32_t) * 4 * n) +
                       align256(sizeof(uint32_t) * 4);
  const size_t o_rank = o_src + align256(sizeof(uint32_t) * 3 * n);
  const size_t o_kind = o_rank + align256(sizeof(uint32_t) * 3 * n);
  const size_t o_bcount = o_kind + align256(3 * (size_t)n);
  uint32_t* src = reinterpret_cast<uint32_t*>(w + o_src);
  uint32_t* rank = reinterpret_cast<uint32_t*>(w + o_rank);
  uint8_t* kind = reinterpret_cast<uint8_t*>(w + o_kind);
  uint32_t* bcount = reinterpret_cast<uint32_t*>(w + o_bcount);
  const int nb = div_up(n, kDensScanBlock);
  DensifyParams d{max_grad, min_opacity, extent, percent_dense, prune_big};
  k_densify_classify<<<div_up(n, 256), 256, 0, st>>>(n, grad_accum, denom, scaling, opacity, d, cls);
  k_densify_block_counts<<<nb, kDensScanBlock, 0, st>>>(n, cls, bcount);
  k_densify_block_prefix<<<1, 1024, 0, st>>>(nb, bcount, tot);
  k_densify_positions<<<nb, kDensScanBlock, 0, st>>>(n, cls, bcount, pos);
  k_densify_map<<<div_up(n, 256), 256, 0, st>>>(n, cls, pos, tot, src, kind, rank);
  uint32_t h[4];
  if (cudaMemcpyAsync(h, tot, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  // kept originals, kept clones, split points, kept children per copy
  for (int b = 0; b < 4; ++b) counts[b] = h[b];
  return CFGS_OK;
}

// Writes one parameter array of the new model from the row map cfgs_densify_plan left in
// `workspace`: rows = counts[0] + counts[1] + 2 counts[3].
// role 0: plain parameter (copied), 1: Adam moment (zero for new rows), 2: xyz, 3: scaling
// (children computed), z = standard-normal draws [2][counts[2]][3] for roles 2 and 3.
extern "C" int cfgs_densify_write(int64_t num_gaussians, void* workspace, const int64_t counts[4], int32_t width,
                                  const float* in, float* out, int32_t role, const float* xyz, const float* scaling,
                                  const float* rotation, const float* z, void* stream) {
  if (num_gaussians <= 0 || !workspace || !counts || width <= 0 || !in || !out || role < 0 || role > 3)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (role >= 2 && (!xyz || !scaling || !rotation || (counts[3] > 0 && !z))) return CFGS_ERR_INVALID_ARGUMENT;
  if ((role == 2 || role == 3) && width != 3) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = num_gaussians;
  char* w = static_cast<char*>(workspace);
  const size_t o_pos = align256(sizeof(uint32_t) * n);
  const size_t o_tot = o_pos + align256(sizeof(uint32_t) * 4 * n);
  const size_t o_src = o_tot + align256(sizeof(uint32_t) * 4);
  const size_t o_rank = o_src + align256(sizeof(uint32_t) * 3 * n);
  const size_t o_kind = o_rank + align256(sizeof(uint32_t) * 3 * n);
  uint32_t* src = reinterpret_cast<uint32_t*>(w + o_src);
  uint32_t* rank = reinterpret_cast<uint32_t*>(w + o_rank);
  uint8_t* kind = reinterpret_cast<uint8_t*>(w + o_kind);
  const int64_t rows = counts[0] + counts[1] + 2 * counts[3];
  if (rows > 3 * n) return CFGS_ERR_INVALID_ARGUMENT;
  if (rows > 0) {
    k_densify_gather<<<div_up(rows * width, 256), 256, 0, st>>>(rows, width, in, out, src, kind, role == 1);
    if (role >= 2 && counts[3] > 0)
      k_densify_children<<<div_up(rows, 256), 256, 0, st>>>(rows, src, kind, rank, (uint32_t)counts[2], xyz, scaling,
                                                           rotation, z, out, role == 3);
  }
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}
