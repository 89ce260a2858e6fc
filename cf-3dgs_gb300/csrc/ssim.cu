// Fused SSIM (structural similarity) with an 11x11 Gaussian window, forward and
// backward, as the CF-3DGS pose loss uses it: utils/loss_utils.py:23-58 and
// trainer/losses.py:147-251 (window sigma 1.5, zero padding 5, one window per channel,
// C1 = 0.01^2, C2 = 0.03^2, mean over every channel and pixel).
//
// Per channel and pixel p the five windowed moments mu1 = W*x, mu2 = W*y, exx = W*x^2,
// eyy = W*y^2, exy = W*xy give
//   S = (2 mu1 mu2 + C1)(2 s12 + C2) / ((mu1^2 + mu2^2 + C1)(s11 + s22 + C2)),
//   s11 = exx - mu1^2, s22 = eyy - mu2^2, s12 = exy - mu1 mu2.
// The forward writes, besides the partial sums of S, the three maps
//   a = dS/dmu1, b = dS/dexx, c = dS/dexy    (times 1/count: d mean / d S_p)
// and the backward forms dL/dx_q = g (W*a + 2 x_q W*b + y_q W*c)_q with g = dL/dmean
// (the window is symmetric, so the transposed convolution is the same convolution).
//
// Both kernels work on 32x32 output tiles of one channel: the tile and a 5-pixel halo
// are staged in shared memory (zero outside the image); a horizontal 11-tap pass over all
// staged rows and then a vertical pass compute runs of 4 outputs per thread, each input
// loaded once per run and the window slid in registers.
#include <cuda.h>  // CUtensorMap and its enumerations (the encoder comes from the runtime)
#include <cudaTypedefs.h>

#include <cmath>

#include "cfgs_internal.cuh"

namespace cfgs {

constexpr int kSsimR = 5;  // window radius
constexpr int kSsimTaps = 2 * kSsimR + 1;
constexpr int kSsimT = 32;                        // output tile: 32 x 32
constexpr int kSsimS = kSsimT + 2 * kSsimR;       // staged rows / columns (42)
constexpr int kSsimSP = 48;  // staged row: columns x0-8 .. x0+39 (a 16-byte-aligned tensor-copy box)
constexpr int kSsimOff = 3;  // staged column of x0 - 5
constexpr uint32_t kSsimBoxBytes = sizeof(float) * kSsimSP * kSsimS;
constexpr int kSsimHP = kSsimT + 1;               // horizontal-result row stride (33)
constexpr int kSsimRun = 4;                       // outputs per thread along a row / column
constexpr int kSsimThreads = 256;
constexpr float kSsimC1 = 0.0001f, kSsimC2 = 0.0009f;

__constant__ float c_ssim_w[kSsimTaps];

// Reciprocal to within one unit in the last place (the loss is held to a tolerance).
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

struct SsimDims {
  int C, H, W, tiles_x, tiles_y;
};

__device__ __forceinline__ float load_or_zero(const float* img, int H, int W, int y, int x) {
  return (y >= 0 && y < H && x >= 0 && x < W) ? img[(size_t)y * W + x] : 0.0f;
}

// One 48 x 42 box of plane z at (x, y) into shared memory by a tensor copy; coordinates
// outside the tensor read as zero.
__device__ __forceinline__ void tma_box(float* dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// Stages `planes` boxes of the tile's rows y0-5 .. y0+36 and columns x0-8 .. x0+39 (zero
// outside the image): by tensor copies (TMA) or by plain loads. Returns false if a
// bounded wait on the copies ran out.
template <bool TMA, int NP>
__device__ __forceinline__ bool stage_planes(float* (&dst)[NP], const float* const (&src)[NP],
                                             const CUtensorMap* const (&maps)[NP], const int (&zidx)[NP], int H,
                                             int W, int x0, int y0, uint64_t* bar_word) {
  if constexpr (TMA) {
    const uint32_t bar = smem_addr(bar_word);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(NP * kSsimBoxBytes)
                   : "memory");
#pragma unroll
      for (int p = 0; p < NP; ++p) tma_box(dst[p], maps[p], x0 - 8, y0 - kSsimR, zidx[p], bar);
    }
    return mbar_wait(bar, 0);
  } else {
    for (int i = threadIdx.x; i < kSsimS * kSsimS; i += kSsimThreads) {
      const int r = i / kSsimS, c = i % kSsimS;
#pragma unroll
      for (int p = 0; p < NP; ++p)
        dst[p][r * kSsimSP + kSsimOff + c] = load_or_zero(src[p], H, W, y0 + r - kSsimR, x0 + c - kSsimR);
    }
    return true;
  }
}

// Block-wide sum of one double per thread (kSsimThreads threads), fixed order.
__device__ __forceinline__ double block_sum_fixed(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kSsimThreads / 32; ++w) t += sh[w];
  return t;  // valid in thread 0
}

// Horizontal 11-tap sums of NQ staged quantities for kSsimRun consecutive outputs of one
// staged row: the 14 inputs are loaded once and the window slides in registers.
// prod(u, v, out) expands two staged values into the NQ quantities.
template <int NQ, class Prod>
__device__ __forceinline__ void hpass_run(const float* a_row, const float* b_row, int c0, float (&out)[NQ][kSsimRun],
                                          Prod prod) {
  float q[kSsimRun + 2 * kSsimR][NQ];
#pragma unroll
  for (int k = 0; k < kSsimRun + 2 * kSsimR; ++k) prod(a_row[c0 + k], b_row ? b_row[c0 + k] : 0.f, q[k]);
#pragma unroll
  for (int u = 0; u < kSsimRun; ++u)
#pragma unroll
    for (int n = 0; n < NQ; ++n) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < kSsimTaps; ++k) acc = fmaf(c_ssim_w[k], q[u + k][n], acc);
      out[n][u] = acc;
    }
}

template <bool TMA>
__global__ void __launch_bounds__(kSsimThreads) k_ssim_fwd(SsimDims d, const float* __restrict__ img1,
                                                           const float* __restrict__ img2, float* __restrict__ maps,
                                                           double* __restrict__ partials, float inv_count,
                                                           const __grid_constant__ CUtensorMap t1,
                                                           const __grid_constant__ CUtensorMap t2) {
  __shared__ __align__(128) float s_x[kSsimS * kSsimSP];
  __shared__ __align__(128) float s_y[kSsimS * kSsimSP];
  __shared__ float s_h[5][kSsimS * kSsimHP];  // horizontal sums of x, y, xx, yy, xy
  __shared__ double s_red[kSsimThreads / 32];
  __shared__ __align__(8) uint64_t s_bar;
  const int tile = blockIdx.x, ch = blockIdx.y;
  const int x0 = (tile % d.tiles_x) * kSsimT, y0 = (tile / d.tiles_x) * kSsimT;
  const size_t plane = (size_t)d.H * d.W;
  float* dst[2] = {s_x, s_y};
  const float* const src[2] = {img1 + ch * plane, img2 + ch * plane};
  const CUtensorMap* const tm[2] = {&t1, &t2};
  const int zi[2] = {ch, ch};
  const bool staged = stage_planes<TMA, 2>(dst, src, tm, zi, d.H, d.W, x0, y0, &s_bar);
  __syncthreads();
  // horizontal: item = (staged row r, run of 4 output columns)
  for (int it = threadIdx.x; it < kSsimS * (kSsimT / kSsimRun); it += kSsimThreads) {
    const int r = it / (kSsimT / kSsimRun), c0 = (it % (kSsimT / kSsimRun)) * kSsimRun;
    float out[5][kSsimRun];
    hpass_run<5>(s_x + r * kSsimSP + kSsimOff, s_y + r * kSsimSP + kSsimOff, c0, out, [](float u, float v, float (&q)[5]) {
      q[0] = u;
      q[1] = v;
      q[2] = u * u;
      q[3] = v * v;
      q[4] = u * v;
    });
#pragma unroll
    for (int n = 0; n < 5; ++n)
#pragma unroll
      for (int u = 0; u < kSsimRun; ++u) s_h[n][r * kSsimHP + c0 + u] = out[n][u];
  }
  __syncthreads();
  // vertical: item = (output column c, run of 4 output rows); one item per thread
  float ssum = 0.f;
  {
    const int c = threadIdx.x % kSsimT, r0 = (threadIdx.x / kSsimT) * kSsimRun;
    float acc[5][kSsimRun];
#pragma unroll
    for (int n = 0; n < 5; ++n)
#pragma unroll
      for (int u = 0; u < kSsimRun; ++u) acc[n][u] = 0.f;
#pragma unroll
    for (int k = 0; k < kSsimRun + 2 * kSsimR; ++k) {
      float v[5];
#pragma unroll
      for (int n = 0; n < 5; ++n) v[n] = s_h[n][(r0 + k) * kSsimHP + c];
#pragma unroll
      for (int u = 0; u < kSsimRun; ++u) {
        const int tap = k - u;
        if (tap >= 0 && tap < kSsimTaps) {
#pragma unroll
          for (int n = 0; n < 5; ++n) acc[n][u] = fmaf(c_ssim_w[tap], v[n], acc[n][u]);
        }
      }
    }
    const int px = x0 + c;
#pragma unroll
    for (int u = 0; u < kSsimRun; ++u) {
      const int py = y0 + r0 + u;
      if (py >= d.H || px >= d.W) continue;
      const float mu1 = acc[0][u], mu2 = acc[1][u], exx = acc[2][u], eyy = acc[3][u], exy = acc[4][u];
      const float m11 = mu1 * mu1, m22 = mu2 * mu2, m12 = mu1 * mu2;
      const float A = 2.f * m12 + kSsimC1, B = 2.f * (exy - m12) + kSsimC2;
      const float Cc = m11 + m22 + kSsimC1, D = (exx - m11) + (eyy - m22) + kSsimC2;
      const float rA = rcp_approx(A), rB = rcp_approx(B), rC = rcp_approx(Cc), rD = rcp_approx(D);
      const float S = (A * B) * (rC * rD);
      ssum += S;
      const size_t q = ch * plane + (size_t)py * d.W + px;
      // dS/dmu1 = S (2 mu2/A - 2 mu2/B - 2 mu1/C + 2 mu1/D); dS/dexx = -S/D; dS/dexy = 2 S/B
      const float da = S * (2.f * mu2 * (rA - rB) + 2.f * mu1 * (rD - rC));
      maps[q] = inv_count * da;
      maps[(size_t)d.C * plane + q] = inv_count * (-S * rD);
      maps[2 * (size_t)d.C * plane + q] = inv_count * (2.f * S * rB);
    }
  }
  const double t = block_sum_fixed((double)ssum, s_red);
  // a copy that did not arrive makes the mean NaN (visibly invalid)
  if (threadIdx.x == 0) partials[(size_t)ch * gridDim.x + tile] = staged ? t : __longlong_as_double(0x7ff8000000000000ll);
}

// Mean SSIM from the per-tile partial sums, in a fixed order (one block).
__global__ void __launch_bounds__(kSsimThreads) k_ssim_mean(const double* __restrict__ partials, int count,
                                                            double inv_count, float* __restrict__ out) {
  __shared__ double s_red[kSsimThreads / 32];
  double v = 0.0;
  for (int i = threadIdx.x; i < count; i += kSsimThreads) v += partials[i];
  const double t = block_sum_fixed(v, s_red);
  if (threadIdx.x == 0) *out = (float)(t * inv_count);
}

template <bool TMA>
__global__ void __launch_bounds__(kSsimThreads) k_ssim_bwd(SsimDims d, const float* __restrict__ img1,
                                                           const float* __restrict__ img2,
                                                           const float* __restrict__ maps,
                                                           const float* __restrict__ dL_dmean,
                                                           float* __restrict__ dL_dimg1,
                                                           const __grid_constant__ CUtensorMap tmaps) {
  __shared__ __align__(128) float s_m[3][kSsimS * kSsimSP];
  __shared__ float s_h[3][kSsimS * kSsimHP];
  __shared__ __align__(8) uint64_t s_bar;
  const int tile = blockIdx.x, ch = blockIdx.y;
  const int x0 = (tile % d.tiles_x) * kSsimT, y0 = (tile / d.tiles_x) * kSsimT;
  const size_t plane = (size_t)d.H * d.W;
  float* dst[3] = {s_m[0], s_m[1], s_m[2]};
  const float* const src[3] = {maps + (size_t)ch * plane, maps + ((size_t)d.C + ch) * plane,
                               maps + (2 * (size_t)d.C + ch) * plane};
  const CUtensorMap* const tm[3] = {&tmaps, &tmaps, &tmaps};
  const int zi[3] = {ch, d.C + ch, 2 * d.C + ch};
  const bool staged = stage_planes<TMA, 3>(dst, src, tm, zi, d.H, d.W, x0, y0, &s_bar);
  __syncthreads();
  for (int it = threadIdx.x; it < kSsimS * (kSsimT / kSsimRun); it += kSsimThreads) {
    const int r = it / (kSsimT / kSsimRun), c0 = (it % (kSsimT / kSsimRun)) * kSsimRun;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      float out[1][kSsimRun];
      hpass_run<1>(s_m[m] + r * kSsimSP + kSsimOff, nullptr, c0, out, [](float u, float, float (&q)[1]) { q[0] = u; });
#pragma unroll
      for (int u = 0; u < kSsimRun; ++u) s_h[m][r * kSsimHP + c0 + u] = out[0][u];
    }
  }
  __syncthreads();
  const float g = *dL_dmean;
  const int c = threadIdx.x % kSsimT, r0 = (threadIdx.x / kSsimT) * kSsimRun;
  float acc[3][kSsimRun];
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int u = 0; u < kSsimRun; ++u) acc[m][u] = 0.f;
#pragma unroll
  for (int k = 0; k < kSsimRun + 2 * kSsimR; ++k) {
    float v[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) v[m] = s_h[m][(r0 + k) * kSsimHP + c];
#pragma unroll
    for (int u = 0; u < kSsimRun; ++u) {
      const int tap = k - u;
      if (tap >= 0 && tap < kSsimTaps) {
#pragma unroll
        for (int m = 0; m < 3; ++m) acc[m][u] = fmaf(c_ssim_w[tap], v[m], acc[m][u]);
      }
    }
  }
  const int px = x0 + c;
#pragma unroll
  for (int u = 0; u < kSsimRun; ++u) {
    const int py = y0 + r0 + u;
    if (py >= d.H || px >= d.W) continue;
    const size_t q = ch * plane + (size_t)py * d.W + px;
    dL_dimg1[q] = staged ? g * (acc[0][u] + 2.f * img1[q] * acc[1][u] + img2[q] * acc[2][u]) : __int_as_float(0x7fc00000);
  }
}

namespace {

// The window (utils/loss_utils.py:23-29: exp(-(x - 5)^2 / (2 sigma^2)), sigma 1.5,
// normalised to sum 1) goes to constant memory once per device.
bool upload_window(cudaStream_t st) {
  constexpr int kMaxDevices = 64;
  static bool done[kMaxDevices] = {};
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return false;
  if (done[dev]) return true;
  double g[kSsimTaps], sum = 0.0;
  for (int k = 0; k < kSsimTaps; ++k) {
    const double t = (double)(k - kSsimR);
    g[k] = std::exp(-t * t / (2.0 * 1.5 * 1.5));
    sum += g[k];
  }
  float w[kSsimTaps];
  for (int k = 0; k < kSsimTaps; ++k) w[k] = (float)(g[k] / sum);
  if (cudaMemcpyToSymbolAsync(c_ssim_w, w, sizeof(w), 0, cudaMemcpyHostToDevice, st) != cudaSuccess) return false;
  if (cudaStreamSynchronize(st) != cudaSuccess) return false;
  done[dev] = true;
  return true;
}

SsimDims dims(int32_t C, int32_t H, int32_t W) {
  SsimDims d;
  d.C = C;
  d.H = H;
  d.W = W;
  d.tiles_x = (W + kSsimT - 1) / kSsimT;
  d.tiles_y = (H + kSsimT - 1) / kSsimT;
  return d;
}

// Rank-3 tensor map of a [D][H][W] float32 array with the staging box (48 x 42 x 1);
// false when the array cannot be described (width not a multiple of 4 floats, base not
// 16-byte aligned) or the encoder is unavailable — the kernels then stage by plain loads.
bool encode_planes(CUtensorMap* m, const float* base, int W, int H, int D) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (!encode || (W % 4) != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
  const cuuint64_t dim[3] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D};
  const cuuint64_t stride[2] = {(cuuint64_t)W * sizeof(float), (cuuint64_t)W * H * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)kSsimSP, (cuuint32_t)kSsimS, 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dim, stride, box, estride,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool dims_ok(int32_t C, int32_t H, int32_t W) {
  return C > 0 && H > 0 && W > 0 && C <= 65535 && (int64_t)C * H * W <= ((int64_t)1 << 31);
}

}  // namespace

}  // namespace cfgs

using namespace cfgs;

extern "C" size_t cfgs_ssim_scratch_bytes(int32_t channels, int32_t height, int32_t width) {
  if (!dims_ok(channels, height, width)) return 0;
  const SsimDims d = dims(channels, height, width);
  const size_t maps = sizeof(float) * 3 * (size_t)channels * height * width;
  const size_t parts = sizeof(double) * (size_t)channels * d.tiles_x * d.tiles_y;
  return align256(maps) + align256(parts);
}

extern "C" int cfgs_ssim_forward(int32_t channels, int32_t height, int32_t width, const float* img1,
                                 const float* img2, void* scratch, float* ssim_mean, void* stream) {
  if (!dims_ok(channels, height, width) || !img1 || !img2 || !scratch || !ssim_mean) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (!upload_window(st)) return CFGS_ERR_LAUNCH;
  const SsimDims d = dims(channels, height, width);
  const size_t count = (size_t)channels * height * width;
  float* maps = static_cast<float*>(scratch);
  double* parts = reinterpret_cast<double*>(static_cast<char*>(scratch) + align256(sizeof(float) * 3 * count));
  const int tiles = d.tiles_x * d.tiles_y;
  CUtensorMap t1{}, t2{};
  const bool tma = encode_planes(&t1, img1, width, height, channels) && encode_planes(&t2, img2, width, height, channels);
  if (tma)
    k_ssim_fwd<true><<<dim3(tiles, channels), kSsimThreads, 0, st>>>(d, img1, img2, maps, parts,
                                                                    (float)(1.0 / (double)count), t1, t2);
  else
    k_ssim_fwd<false><<<dim3(tiles, channels), kSsimThreads, 0, st>>>(d, img1, img2, maps, parts,
                                                                     (float)(1.0 / (double)count), t1, t2);
  k_ssim_mean<<<1, kSsimThreads, 0, st>>>(parts, tiles * channels, 1.0 / (double)count, ssim_mean);
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}

extern "C" int cfgs_ssim_backward(int32_t channels, int32_t height, int32_t width, const float* img1,
                                  const float* img2, const void* scratch, const float* dL_dmean, float* dL_dimg1,
                                  void* stream) {
  if (!dims_ok(channels, height, width) || !img1 || !img2 || !scratch || !dL_dmean || !dL_dimg1)
    return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (!upload_window(st)) return CFGS_ERR_LAUNCH;
  const SsimDims d = dims(channels, height, width);
  const float* maps = static_cast<const float*>(scratch);
  CUtensorMap tm{};
  const dim3 grid(d.tiles_x * d.tiles_y, channels);
  if (encode_planes(&tm, maps, width, height, 3 * channels))
    k_ssim_bwd<true><<<grid, kSsimThreads, 0, st>>>(d, img1, img2, maps, dL_dmean, dL_dimg1, tm);
  else
    k_ssim_bwd<false><<<grid, kSsimThreads, 0, st>>>(d, img1, img2, maps, dL_dmean, dL_dimg1, tm);
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}
