// Forward phase 1: per-Gaussian preprocess (EWA projection, SH colour, radius, tile
// rectangle), per-tile instance counts and the two scans. Also markVisible.
//
// This translation unit is compiled with -fmad=false: every a*b+c below is two
// IEEE-rounded operations unless written as fmaf(), so the CPU oracle reproduces the
// outputs (radii, rectangles, depth keys, conics) bit for bit.
//
// Algorithm: the published 3DGS preprocess (EWA splatting, Zwicker et al. 2001, with
// the 3DGS low-pass of 0.3 px^2 and the 1.3*tan(fov) Jacobian clamp), restated. The
// reference's Python statements of the same math are utils/general_utils.py:76-108
// (covariance), utils/sh_utils.py:57-112 (SH), scene/cameras.py:57-74 and
// utils/graphics_utils.py:85-113 (camera matrices).
#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

struct CamConst {
  float V[16];
  float P[16];
  float campos[3];
};

__device__ __forceinline__ void load_cam(const CfgsSettings& s, CamConst& c) {
#pragma unroll
  for (int i = 0; i < 16; ++i) c.V[i] = __ldg(s.viewmatrix + i);
#pragma unroll
  for (int i = 0; i < 16; ++i) c.P[i] = __ldg(s.projmatrix + i);
  if (s.campos) {
    c.campos[0] = __ldg(s.campos + 0);
    c.campos[1] = __ldg(s.campos + 1);
    c.campos[2] = __ldg(s.campos + 2);
  } else {
    c.campos[0] = c.campos[1] = c.campos[2] = 0.f;
  }
}

// [p,1] @ M, columns 0..2 (row-vector convention of the stored matrices).
__device__ __forceinline__ float3 xform43(const float* m, float3 p) {
  float3 r;
  r.x = fmaf(m[8], p.z, fmaf(m[4], p.y, fmaf(m[0], p.x, m[12])));
  r.y = fmaf(m[9], p.z, fmaf(m[5], p.y, fmaf(m[1], p.x, m[13])));
  r.z = fmaf(m[10], p.z, fmaf(m[6], p.y, fmaf(m[2], p.x, m[14])));
  return r;
}
__device__ __forceinline__ float xform_w(const float* m, float3 p) {
  return fmaf(m[11], p.z, fmaf(m[7], p.y, fmaf(m[3], p.x, m[15])));
}

// Sigma = R diag(s)^2 R^T with R the rotation of quaternion (r,x,y,z) (not
// normalised here; CF-3DGS normalises in Python), stored (xx,xy,xz,yy,yz,zz).
__device__ __forceinline__ void cov3d_from_scale_rot(float3 s, float mod, float4 q, float* cov) {
  float sx = mod * s.x, sy = mod * s.y, sz = mod * s.z;
  float r = q.x, x = q.y, y = q.z, z = q.w;
  float xx = x * x, yy = y * y, zz = z * z;
  float xy = x * y, xz = x * z, yz = y * z;
  float rx = r * x, ry = r * y, rz = r * z;
  float R[9];
  R[0] = 1.0f - 2.0f * (yy + zz);
  R[1] = 2.0f * (xy - rz);
  R[2] = 2.0f * (xz + ry);
  R[3] = 2.0f * (xy + rz);
  R[4] = 1.0f - 2.0f * (xx + zz);
  R[5] = 2.0f * (yz - rx);
  R[6] = 2.0f * (xz - ry);
  R[7] = 2.0f * (yz + rx);
  R[8] = 1.0f - 2.0f * (xx + yy);
  float M[9];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    M[3 * i + 0] = R[3 * i + 0] * sx;
    M[3 * i + 1] = R[3 * i + 1] * sy;
    M[3 * i + 2] = R[3 * i + 2] * sz;
  }
  const int ii[6] = {0, 0, 0, 1, 1, 2};
  const int jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const float* a = M + 3 * ii[k];
    const float* b = M + 3 * jj[k];
    cov[k] = fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0]));
  }
}

// 2D screen covariance (a, b, c) = J W Sigma W^T J^T + 0.3 I.
__device__ __forceinline__ float3 cov2d(float3 t, float fx, float fy, float tanfovx, float tanfovy,
                                        const float* cov, const float* V) {
  float limx = 1.3f * tanfovx;
  float limy = 1.3f * tanfovy;
  float txtz = t.x / t.z;
  float tytz = t.y / t.z;
  float tx = fminf(limx, fmaxf(-limx, txtz)) * t.z;
  float ty = fminf(limy, fmaxf(-limy, tytz)) * t.z;
  float tz2 = t.z * t.z;
  float J00 = fx / t.z;
  float J02 = -(fx * tx) / tz2;
  float J11 = fy / t.z;
  float J12 = -(fy * ty) / tz2;
  // W[i][j] = V[4j+i]; rows of T = J W.
  float T0[3], T1[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    T0[j] = fmaf(J02, V[4 * j + 2], J00 * V[4 * j + 0]);
    T1[j] = fmaf(J12, V[4 * j + 2], J11 * V[4 * j + 1]);
  }
  float S[9] = {cov[0], cov[1], cov[2], cov[1], cov[3], cov[4], cov[2], cov[4], cov[5]};
  float u[3], v[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    u[i] = fmaf(S[3 * i + 2], T0[2], fmaf(S[3 * i + 1], T0[1], S[3 * i + 0] * T0[0]));
    v[i] = fmaf(S[3 * i + 2], T1[2], fmaf(S[3 * i + 1], T1[1], S[3 * i + 0] * T1[0]));
  }
  float a = fmaf(T0[2], u[2], fmaf(T0[1], u[1], T0[0] * u[0]));
  float b = fmaf(T0[2], v[2], fmaf(T0[1], v[1], T0[0] * v[0]));
  float c = fmaf(T1[2], v[2], fmaf(T1[1], v[1], T1[0] * v[0]));
  return make_float3(a + 0.3f, b, c + 0.3f);
}

__device__ __forceinline__ float ndc2pix(float v, int S) { return ((v + 1.0f) * (float)S - 1.0f) * 0.5f; }

// Colour from real SH of degree <= 3 at the view direction, + 0.5, clamped at 0.
__device__ __forceinline__ float3 sh_to_rgb(int deg, const float* sh, float3 p, const float* campos,
                                            uint8_t* clamped, bool vec16) {
  float dx = p.x - campos[0], dy = p.y - campos[1], dz = p.z - campos[2];
  float len = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
  float x = dx / len, y = dy / len, z = dz / len;
  float b[kMaxShCoeffs];
  b[0] = CFGS_SH_C0;
  int nb = 1;
  if (deg > 0) {
    b[1] = -CFGS_SH_C1 * y;
    b[2] = CFGS_SH_C1 * z;
    b[3] = -CFGS_SH_C1 * x;
    nb = 4;
    if (deg > 1) {
      float xx = x * x, yy = y * y, zz = z * z;
      float xy = x * y, yz = y * z, xz = x * z;
      b[4] = CFGS_SH_C2_0 * xy;
      b[5] = CFGS_SH_C2_1 * yz;
      b[6] = CFGS_SH_C2_2 * ((2.0f * zz - xx) - yy);
      b[7] = CFGS_SH_C2_3 * xz;
      b[8] = CFGS_SH_C2_4 * (xx - yy);
      nb = 9;
      if (deg > 2) {
        b[9] = (CFGS_SH_C3_0 * y) * (3.0f * xx - yy);
        b[10] = (CFGS_SH_C3_1 * xy) * z;
        b[11] = (CFGS_SH_C3_2 * y) * ((4.0f * zz - xx) - yy);
        b[12] = (CFGS_SH_C3_3 * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
        b[13] = (CFGS_SH_C3_4 * x) * ((4.0f * zz - xx) - yy);
        b[14] = (CFGS_SH_C3_5 * z) * (xx - yy);
        b[15] = (CFGS_SH_C3_6 * x) * (xx - 3.0f * yy);
        nb = 16;
      }
    }
  }
  float r, g, bl;
  if (nb == kMaxShCoeffs && vec16) {
    // 16 coefficients, 16-byte aligned: 12 float4 loads, consumed in the same
    // (coefficient, channel) order as the scalar path below
    const float4* s4 = reinterpret_cast<const float4*>(sh);
    float c[3];
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      const float4 f = s4[q];
      const float e[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = (4 * q + u) / 3, ch = (4 * q + u) % 3;
        c[ch] = k == 0 ? b[0] * e[u] : fmaf(b[k], e[u], c[ch]);
      }
    }
    r = c[0];
    g = c[1];
    bl = c[2];
  } else {
    r = b[0] * sh[0];
    g = b[0] * sh[1];
    bl = b[0] * sh[2];
#pragma unroll
    for (int k = 1; k < kMaxShCoeffs; ++k) {
      if (k < nb) {
        r = fmaf(b[k], sh[3 * k + 0], r);
        g = fmaf(b[k], sh[3 * k + 1], g);
        bl = fmaf(b[k], sh[3 * k + 2], bl);
      }
    }
  }
  r = r + 0.5f;
  g = g + 0.5f;
  bl = bl + 0.5f;
  *clamped = (uint8_t)((r < 0.0f ? 1 : 0) | (g < 0.0f ? 2 : 0) | (bl < 0.0f ? 4 : 0));
  return make_float3(fmaxf(r, 0.0f), fmaxf(g, 0.0f), fmaxf(bl, 0.0f));
}

__device__ __forceinline__ uint32_t block_reduce_sum_u32(uint32_t v, uint32_t* sh_warp) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh_warp[warp] = v;
  __syncthreads();
  uint32_t t = 0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh_warp[w];
  }
  return t;  // valid in thread 0
}

template <class Scenes>
__global__ void __launch_bounds__(kPreprocessBlock) k_preprocess(PreArgs<Scenes> a) {
  __shared__ uint32_t sh_warp[kPreprocessBlock / 32];
  const SceneDesc& sd = a.scenes.for_block(blockIdx.x);
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = idx - sd.gauss_base < sd.num_gaussians;
  uint32_t touched = 0;
  if (valid) {
    int radius = 0;
    float V[16], P[16], campos[3];
#pragma unroll
    for (int i = 0; i < 16; ++i) V[i] = __ldg(sd.V + i);
#pragma unroll
    for (int i = 0; i < 16; ++i) P[i] = __ldg(sd.P + i);
    campos[0] = sd.campos ? __ldg(sd.campos + 0) : 0.f;
    campos[1] = sd.campos ? __ldg(sd.campos + 1) : 0.f;
    campos[2] = sd.campos ? __ldg(sd.campos + 2) : 0.f;
    if (a.g.shs) {  // the SH lines are read only after the projection: ask L2 for them now
      const char* shp = reinterpret_cast<const char*>(a.g.shs + (size_t)idx * sd.sh_coeffs * 3);
      const int bytes = sd.sh_coeffs * 3 * (int)sizeof(float);
      for (int o = 0; o < bytes; o += 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(shp + o));
    }
    float3 p = posed_mean(sd, a.g.means3D, (size_t)idx);
    float3 t = xform43(V, p);
    bool culled = t.z <= CFGS_NEAR_Z;
    if (culled && sd.prefiltered) atomicOr(&a.counts->flags, CFGS_FLAG_FRUSTUM_VIOLATION);
    if (!culled) {
      float3 hom = xform43(P, p);
      float hw = xform_w(P, p);
      float w_inv = 1.0f / (hw + 0.0000001f);
      float3 proj = make_float3(hom.x * w_inv, hom.y * w_inv, hom.z * w_inv);
      float cov[6];
      if (a.g.cov3D_precomp) {
        const float* c = a.g.cov3D_precomp + 6 * (size_t)idx;
#pragma unroll
        for (int k = 0; k < 6; ++k) cov[k] = c[k];
      } else {
        const float* s = a.g.scales + 3 * (size_t)idx;
        const float* qp = a.g.rotations + 4 * (size_t)idx;
        float4 q = make_float4(qp[0], qp[1], qp[2], qp[3]);
        cov3d_from_scale_rot(make_float3(s[0], s[1], s[2]), sd.scale_modifier, q, cov);
      }
      float3 c2 = cov2d(t, sd.focal_x, sd.focal_y, sd.tanfovx, sd.tanfovy, cov, V);
      float det = c2.x * c2.z - c2.y * c2.y;
      if (det != 0.0f) {
        float det_inv = 1.0f / det;
        float3 conic = make_float3(c2.z * det_inv, -c2.y * det_inv, c2.x * det_inv);
        float mid = 0.5f * (c2.x + c2.z);
        float disc = sqrtf(fmaxf(0.1f, mid * mid - det));
        float l1 = mid + disc, l2 = mid - disc;
        float rad_f = ceilf(3.0f * sqrtf(fmaxf(l1, l2)));
        int rad = (int)rad_f;
        float2 pimg = make_float2(ndc2pix(proj.x, sd.W), ndc2pix(proj.y, sd.H));
        float rf = (float)rad;
        int rminx = min(sd.grid_x, max(0, (int)((pimg.x - rf) / (float)kTileX)));
        int rminy = min(sd.grid_y, max(0, (int)((pimg.y - rf) / (float)kTileY)));
        int rmaxx = min(sd.grid_x, max(0, (int)(((pimg.x + rf) + (float)(kTileX - 1)) / (float)kTileX)));
        int rmaxy = min(sd.grid_y, max(0, (int)(((pimg.y + rf) + (float)(kTileY - 1)) / (float)kTileY)));
        uint32_t area = (uint32_t)((rmaxx - rminx) * (rmaxy - rminy));
        if (area > 0) {
          float3 rgb;
          uint8_t cl = 0;
          if (a.g.colors_precomp) {
            const float* c = a.g.colors_precomp + 3 * (size_t)idx;
            rgb = make_float3(c[0], c[1], c[2]);
          } else {
            const float* shp = a.g.shs + (size_t)idx * sd.sh_coeffs * 3;
            rgb = sh_to_rgb(sd.sh_degree, shp, p, campos, &cl,
                            sd.sh_coeffs == kMaxShCoeffs && (((uintptr_t)shp) & 15) == 0);
          }
          a.geom.xy[idx] = pimg;
          a.geom.conic_op[idx] = make_float4(conic.x, conic.y, conic.z, a.g.opacities[idx]);
          a.geom.rgbd[idx] = make_float4(rgb.x, rgb.y, rgb.z, t.z);
          a.geom.rect[idx] = make_uint2((uint32_t)rminx | ((uint32_t)rminy << 16),
                                        (uint32_t)rmaxx | ((uint32_t)rmaxy << 16));
          a.geom.clamped[idx] = cl;
          touched = area;
          radius = rad;
        }
      }
    }
    a.radii[idx] = radius;
  }
  if (idx < a.total_slots) {
    a.geom.touched[idx] = touched;
    if (!valid) a.radii[idx] = 0;
  }
  uint32_t bs = block_reduce_sum_u32(touched, sh_warp);
  if (threadIdx.x == 0) a.geom.block_sums[blockIdx.x] = bs;
}

template <class Scenes>
void launch_preprocess(const PreArgs<Scenes>& a, int blocks, cudaStream_t st) {
  k_preprocess<Scenes><<<blocks, kPreprocessBlock, 0, st>>>(a);
}
template void launch_preprocess<SingleScene>(const PreArgs<SingleScene>&, int, cudaStream_t);
template void launch_preprocess<SceneTable>(const PreArgs<SceneTable>&, int, cudaStream_t);

// Instance count K = sum of the per-block touched sums (one block of 1024 threads).
__global__ void __launch_bounds__(1024) k_scan(const uint32_t* block_sums, int num_blocks, CfgsCounts* counts) {
  __shared__ unsigned long long sh[32];
  unsigned long long v = 0;
  for (int i = threadIdx.x; i < num_blocks; i += blockDim.x) v += block_sums[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long K = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) K += sh[w];
    counts->num_rendered = K > 0xffffffffull ? 0xffffffffu : (uint32_t)K;
    if (K > 0x7fffffffull) atomicOr(&counts->flags, CFGS_FLAG_CAPACITY_OVERFLOW);
  }
}

__global__ void __launch_bounds__(256) k_mark_visible(int n, const float* means, const float* V,
                                                      uint8_t* vis) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float m[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) m[k] = __ldg(V + k);
  float3 p = make_float3(means[3 * i], means[3 * i + 1], means[3 * i + 2]);
  float3 t = xform43(m, p);
  vis[i] = t.z <= CFGS_NEAR_Z ? 0 : 1;
}

void launch_scan(uint32_t* block_sums, int num_blocks, CfgsCounts* counts, cudaStream_t st) {
  k_scan<<<1, 1024, 0, st>>>(block_sums, num_blocks, counts);
}

}  // namespace cfgs

using namespace cfgs;

extern "C" size_t cfgs_geom_bytes(int32_t n) { return n < 0 ? 0 : GeomLayout(n).total; }
extern "C" size_t cfgs_image_bytes(int32_t w, int32_t h) {
  return (w <= 0 || h <= 0) ? 0 : ImageLayout(w, h).total;
}
extern "C" size_t cfgs_binning_bytes(int64_t cap) { return cap < 0 ? 0 : BinningLayout(cap).total; }
extern "C" size_t cfgs_backward_scratch_bytes(int64_t cap) {
  return ScratchLayout(cap).total;
}

extern "C" void cfgs_geom_layout(int32_t n, size_t o[14]) {
  GeomLayout L(n < 0 ? 0 : n);
  size_t v[14] = {L.xy,        L.conic_op,  L.rgbd,         L.rect,         L.touched,
                  L.offset,    L.clamped,   L.block_sums,   L.depth_key,    L.depth_val,
                  L.rank_sums, L.depth_counts, L.depth_totals, L.total};
  for (int i = 0; i < 14; ++i) o[i] = v[i];
}
extern "C" void cfgs_image_layout(int32_t w, int32_t h, size_t o[6]) {
  ImageLayout L(w < 1 ? 1 : w, h < 1 ? 1 : h);
  size_t v[6] = {L.header, L.tile_count, L.tile_range, L.final_T, L.n_contrib, L.total};
  for (int i = 0; i < 6; ++i) o[i] = v[i];
}

static bool settings_ok(const CfgsSettings* s) {
  return s && s->image_width > 0 && s->image_height > 0 && s->viewmatrix && s->projmatrix &&
         s->bg && s->sh_degree >= 0 && s->sh_degree <= 3 && s->image_width <= 65535 * kTileX &&
         s->image_height <= 65535 * kTileY;
}

extern "C" int cfgs_preprocess_forward(const CfgsSettings* s, const CfgsGaussians* g, void* geom,
                                       void* image, int32_t* radii, void* stream) {
  if (!settings_ok(s) || !g || !geom || !image) return CFGS_ERR_INVALID_ARGUMENT;
  if (g->num_gaussians < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (g->num_gaussians > 0) {
    if (!g->means3D || !g->opacities || !radii) return CFGS_ERR_INVALID_ARGUMENT;
    if ((g->shs == nullptr) == (g->colors_precomp == nullptr)) return CFGS_ERR_INVALID_ARGUMENT;
    if (g->cov3D_precomp == nullptr && (g->scales == nullptr || g->rotations == nullptr))
      return CFGS_ERR_INVALID_ARGUMENT;
    if (g->shs && g->sh_coeffs < (s->sh_degree + 1) * (s->sh_degree + 1)) return CFGS_ERR_INVALID_ARGUMENT;
    if (g->shs && !s->campos) return CFGS_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  ImageLayout IL(s->image_width, s->image_height);
  ImageView iv(image, s->image_width, s->image_height);
  GeomView gv(geom, g->num_gaussians);
  GeomLayout GL(g->num_gaussians);
  if (cudaMemsetAsync(iv.counts, 0, sizeof(CfgsCounts), st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  if (cudaMemsetAsync(iv.tile_count, 0, sizeof(uint32_t) * IL.num_tiles, st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  if (g->num_gaussians > 0) {
    PreArgs<SingleScene> a;
    a.scenes.d = single_scene_desc(s, g->num_gaussians, g->sh_coeffs);
    a.g = *g;
    a.geom = gv;
    a.counts = iv.counts;
    a.radii = radii;
    a.total_slots = g->num_gaussians;
    k_preprocess<SingleScene><<<GL.num_blocks, kPreprocessBlock, 0, st>>>(a);
    CFGS_CHECK_LAUNCH(s->debug, st);
  }
  launch_scan(gv.block_sums, GL.num_blocks, iv.counts, st);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_read_counts(const void* image, CfgsCounts* out, void* stream) {
  if (!image || !out) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(out, image, sizeof(CfgsCounts), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  if (cudaStreamSynchronize(st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  return CFGS_OK;
}

extern "C" int cfgs_mark_visible(int32_t n, const float* means3D, const float* viewmatrix,
                                 const float* projmatrix, uint8_t* visible, void* stream) {
  (void)projmatrix;
  if (n < 0 || (n > 0 && (!means3D || !viewmatrix || !visible))) return CFGS_ERR_INVALID_ARGUMENT;
  if (n == 0) return CFGS_OK;
  k_mark_visible<<<div_up(n, 256), 256, 0, (cudaStream_t)stream>>>(n, means3D, viewmatrix, visible);
  CFGS_CHECK_LAUNCH(0, stream);
  return CFGS_OK;
}
