// L1 photometric loss, forward and backward: mean |x - t| over every element
// (utils/loss_utils.py:15-16, trainer/losses.py:139-140), optionally of clamp(x, 0, 1) —
// the pose solve clamps the render before its loss (scene/gaussian_model_cf.py:885).
//
// The sum runs over a partition fixed by n and the operands' alignment: a grid of at
// most kL1MaxBlocks blocks, a fixed order inside each block, and a float64 fold of the
// block partials in block order, so repeated calls give the same bits. The gradient is
// the one autograd forms for clamp -> sub -> abs -> mean:
//   dL/dx = (0 <= x <= 1 or no clamp) ? (g * (1 / n)) * sign(c - t) : 0
// (torch divides by the element count through a multiplication by its reciprocal).
// The forward can also write that gradient for g = 1 in the same pass (a loss that ends
// the graph), which reads the operands once.
#include "cfgs_internal.cuh"

namespace cfgs {

constexpr int kL1Threads = 256;
constexpr int kL1MaxBlocks = 4 * 152;  // 4 resident blocks of 8 warps on each of 152 SMs

__device__ __forceinline__ float l1_value(float x, float t, bool clamp) {
  const float c = clamp ? fminf(fmaxf(x, 0.0f), 1.0f) : x;
  return fabsf(c - t);
}

// gn = g * (1 / n); the sign of c - t times gn, masked by the clamp's pass-through range.
__device__ __forceinline__ float l1_grad_value(float x, float t, bool clamp, float gn) {
  const float c = clamp ? fminf(fmaxf(x, 0.0f), 1.0f) : x;
  const float d = c - t;
  const float s = d > 0.0f ? gn : (d < 0.0f ? -gn : 0.0f);
  return (!clamp || (x >= 0.0f && x <= 1.0f)) ? s : 0.0f;
}

__device__ __forceinline__ float block_sum(float v, float* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.0f;
  if (threadIdx.x == 0)
    for (int w = 0; w < kL1Threads / 32; ++w) s += sh[w];
  return s;
}

// Block b covers the units b * 256 + tid + k * (grid * 256): float4 units when VEC (both
// operands and the gradient 16-byte aligned), single floats otherwise; with VEC the last
// n % 4 elements go to block 0's first threads.
template <bool CLAMP, bool VEC>
__global__ void __launch_bounds__(kL1Threads) k_l1_forward(int64_t n, const float* __restrict__ x,
                                                           const float* __restrict__ t, float* __restrict__ partial,
                                                           float* __restrict__ dx, float gn) {
  __shared__ float sh[kL1Threads / 32];
  const int64_t stride = (int64_t)gridDim.x * kL1Threads;
  const int64_t i0 = (int64_t)blockIdx.x * kL1Threads + threadIdx.x;
  float acc = 0.0f;
  if (VEC) {
    const int64_t n4 = n >> 2;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const float4* t4 = reinterpret_cast<const float4*>(t);
    float4* d4 = reinterpret_cast<float4*>(dx);
#pragma unroll 2
    for (int64_t i = i0; i < n4; i += stride) {
      const float4 a = __ldcs(x4 + i), b = __ldcs(t4 + i);
      acc += l1_value(a.x, b.x, CLAMP);
      acc += l1_value(a.y, b.y, CLAMP);
      acc += l1_value(a.z, b.z, CLAMP);
      acc += l1_value(a.w, b.w, CLAMP);
      if (dx)
        __stcs(d4 + i, make_float4(l1_grad_value(a.x, b.x, CLAMP, gn), l1_grad_value(a.y, b.y, CLAMP, gn),
                                   l1_grad_value(a.z, b.z, CLAMP, gn), l1_grad_value(a.w, b.w, CLAMP, gn)));
    }
    const int64_t j = 4 * n4 + i0;
    if (j < n) {
      acc += l1_value(x[j], t[j], CLAMP);
      if (dx) dx[j] = l1_grad_value(x[j], t[j], CLAMP, gn);
    }
  } else {
    for (int64_t i = i0; i < n; i += stride) {
      const float a = x[i], b = t[i];
      acc += l1_value(a, b, CLAMP);
      if (dx) dx[i] = l1_grad_value(a, b, CLAMP, gn);
    }
  }
  const float s = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// One block: the partials summed in float64 in a fixed order, divided by n.
__global__ void __launch_bounds__(kL1Threads) k_l1_fold(const float* __restrict__ partial, int blocks, int64_t n,
                                                        float* __restrict__ loss) {
  __shared__ double sh[kL1Threads];
  double s = 0.0;
  for (int b = threadIdx.x; b < blocks; b += kL1Threads) s += (double)partial[b];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kL1Threads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = (float)(sh[0] / (double)n);
}

template <bool CLAMP, bool VEC>
__global__ void __launch_bounds__(kL1Threads) k_l1_backward(int64_t n, const float* __restrict__ x,
                                                            const float* __restrict__ t,
                                                            const float* __restrict__ g_loss, float* __restrict__ dx) {
  const float gn = __ldg(g_loss) * __frcp_rn((float)n);  // g * (1 / n), as torch's scalar division
  const int64_t stride = (int64_t)gridDim.x * kL1Threads;
  const int64_t i0 = (int64_t)blockIdx.x * kL1Threads + threadIdx.x;
  if (VEC) {
    const int64_t n4 = n >> 2;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const float4* t4 = reinterpret_cast<const float4*>(t);
    float4* d4 = reinterpret_cast<float4*>(dx);
#pragma unroll 2
    for (int64_t i = i0; i < n4; i += stride) {
      const float4 a = __ldcs(x4 + i), b = __ldcs(t4 + i);
      __stcs(d4 + i, make_float4(l1_grad_value(a.x, b.x, CLAMP, gn), l1_grad_value(a.y, b.y, CLAMP, gn),
                                 l1_grad_value(a.z, b.z, CLAMP, gn), l1_grad_value(a.w, b.w, CLAMP, gn)));
    }
    const int64_t j = 4 * n4 + i0;
    if (j < n) dx[j] = l1_grad_value(x[j], t[j], CLAMP, gn);
  } else {
    for (int64_t i = i0; i < n; i += stride) dx[i] = l1_grad_value(x[i], t[i], CLAMP, gn);
  }
}

static bool aligned16(const void* p) { return p == nullptr || (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

static int l1_blocks(int64_t n, bool vec) {
  const int64_t units = vec ? (n >> 2) : n;
  const int64_t b = (units + kL1Threads - 1) / kL1Threads;
  return (int)(b < 1 ? 1 : (b > kL1MaxBlocks ? kL1MaxBlocks : b));
}

}  // namespace cfgs

using namespace cfgs;

extern "C" size_t cfgs_l1_loss_scratch_bytes(int64_t n) {
  (void)n;
  return sizeof(float) * kL1MaxBlocks;
}

extern "C" int cfgs_l1_loss_forward(int64_t n, const float* x, const float* target, int32_t clamp, void* scratch,
                                    float* loss, float* dL_dx, void* stream) {
  if (n < 0 || !loss || !scratch || (n > 0 && (!x || !target))) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  float* partial = static_cast<float*>(scratch);
  int blocks = 0;
  if (n > 0) {
    const bool vec = aligned16(x) && aligned16(target) && aligned16(dL_dx);
    blocks = l1_blocks(n, vec);
    const float gn = 1.0f / (float)n;  // IEEE-rounded, as __frcp_rn on the device
    if (clamp) {
      if (vec) k_l1_forward<true, true><<<blocks, kL1Threads, 0, st>>>(n, x, target, partial, dL_dx, gn);
      else k_l1_forward<true, false><<<blocks, kL1Threads, 0, st>>>(n, x, target, partial, dL_dx, gn);
    } else {
      if (vec) k_l1_forward<false, true><<<blocks, kL1Threads, 0, st>>>(n, x, target, partial, dL_dx, gn);
      else k_l1_forward<false, false><<<blocks, kL1Threads, 0, st>>>(n, x, target, partial, dL_dx, gn);
    }
  }
  k_l1_fold<<<1, kL1Threads, 0, st>>>(partial, blocks, n, loss);  // n = 0: 0 / 0 = NaN, as torch's mean
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}

extern "C" int cfgs_l1_loss_backward(int64_t n, const float* x, const float* target, int32_t clamp,
                                     const float* dL_dloss, float* dL_dx, void* stream) {
  if (n < 0 || (n > 0 && (!x || !target || !dL_dloss || !dL_dx))) return CFGS_ERR_INVALID_ARGUMENT;
  if (n == 0) return CFGS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const bool vec = aligned16(x) && aligned16(target) && aligned16(dL_dx);
  const int blocks = l1_blocks(n, vec);
  if (clamp) {
    if (vec) k_l1_backward<true, true><<<blocks, kL1Threads, 0, st>>>(n, x, target, dL_dloss, dL_dx);
    else k_l1_backward<true, false><<<blocks, kL1Threads, 0, st>>>(n, x, target, dL_dloss, dL_dx);
  } else {
    if (vec) k_l1_backward<false, true><<<blocks, kL1Threads, 0, st>>>(n, x, target, dL_dloss, dL_dx);
    else k_l1_backward<false, false><<<blocks, kL1Threads, 0, st>>>(n, x, target, dL_dloss, dL_dx);
  }
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}
