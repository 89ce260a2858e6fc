// Backward: per-tile render backward with in-block gradient reduction, then the
// per-Gaussian preprocess backward (conic -> 2D covariance -> 3D covariance ->
// scale/rotation, projection -> mean, SH -> coefficients and view direction).
//
// Upstream accumulates every (pixel, Gaussian) gradient with a global atomicAdd.
// Here each tile reduces the gradients of its 256 pixels per instance inside the
// block (a transposing warp reduction, then a fixed-order sum over the 8 warps) and
// writes one 48-byte record per (Gaussian, tile) instance, at the instance's
// pre-sort index. A Gaussian's instances are contiguous in pre-sort order, so the
// preprocess backward sums its records in a fixed order: no atomics, bit-identical
// results run to run.
#include <mutex>

#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

constexpr int kBwdBatch = 64;
constexpr int kWarps = kTilePixels / 32;

// Sums 16 per-lane values across the warp in 16 shuffles (instead of 80): each step
// halves the number of values a lane carries. On return lane L holds the warp total
// of value index L >> 1.
__device__ __forceinline__ float warp_transpose_reduce16(float (&v)[16], int lane) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    bool up = lane & 16;
    float send = up ? v[k] : v[k + 8];
    float keep = up ? v[k + 8] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    bool up = lane & 8;
    float send = up ? v[k] : v[k + 4];
    float keep = up ? v[k + 4] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    bool up = lane & 4;
    float send = up ? v[k] : v[k + 2];
    float keep = up ? v[k + 2] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  {
    bool up = lane & 2;
    float send = up ? v[0] : v[1];
    float keep = up ? v[1] : v[0];
    v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
  return v[0];
}

// d/dc of mean |clamp(c, 0, 1) - t| as autograd forms it.
__device__ __forceinline__ float l1_grad(float c, float t, float inv_numel) {
  float d = fminf(fmaxf(c, 0.0f), 1.0f) - t;
  float sgn = d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f);
  return (c >= 0.0f && c <= 1.0f) ? inv_numel * sgn : 0.0f;
}

// Same pixel boxes and exact shortcuts as the forward (box_may_contribute per warp and
// instance, alpha_threshold per pixel); the cross-warp sum of an instance adds only the
// warps that kept it (the others' terms are exact zeros).
template <class Scenes>
__global__ void __launch_bounds__(kTilePixels) k_render_bwd(RenderBwdArgs<Scenes> a) {
  __shared__ float4 s_xyt[kBwdBatch];
  __shared__ float4 s_co[kBwdBatch];
  __shared__ float4 s_rgbd[kBwdBatch];
  __shared__ uint32_t s_pidx[kBwdBatch];
  __shared__ float s_part[kWarps][kBwdBatch][10];
  __shared__ uint32_t s_keep[kWarps][kBwdBatch / 32];
  __shared__ uint32_t s_max;
  if ((int64_t)a.counts->num_rendered > a.cap) return;
  const int tile = blockIdx.x;
  const SceneDesc& sd = a.scenes.for_tile(tile);
  const int lt = tile - sd.tile_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bx0 = (lt % sd.grid_x) * kTileX + (warp & 1) * 8;
  const int by0 = (lt / sd.grid_x) * kTileY + (warp >> 1) * 4;
  const int px = bx0 + (lane & 7), py = by0 + (lane >> 3);
  const float bxf0 = (float)bx0, bxf1 = (float)(bx0 + 7), byf0 = (float)by0, byf1 = (float)(by0 + 3);
  const bool inside = px < sd.W && py < sd.H;
  const float pxf = (float)px, pyf = (float)py;
  const uint32_t lo = a.tile_range[tile];
  const int n = (int)(a.tile_range[tile + 1] - lo);
  const size_t HW = (size_t)sd.W * sd.H;
  const size_t pix = inside ? (size_t)py * sd.W + px : 0;
  const size_t gp = (size_t)sd.pix_base + pix;

  float T_final = 1.0f, dC0 = 0.f, dC1 = 0.f, dC2 = 0.f, dD = 0.f, dA = 0.f;
  uint32_t last = 0;
  if (inside) {
    T_final = a.final_T[gp];
    last = a.n_contrib[gp];
    const size_t cb = 3 * (size_t)sd.pix_base + pix;
    if (a.target) {
      dC0 = l1_grad(a.color[cb], a.target[cb], sd.inv_numel);
      dC1 = l1_grad(a.color[cb + HW], a.target[cb + HW], sd.inv_numel);
      dC2 = l1_grad(a.color[cb + 2 * HW], a.target[cb + 2 * HW], sd.inv_numel);
    } else {
      dC0 = a.dL_dcolor[cb];
      dC1 = a.dL_dcolor[cb + HW];
      dC2 = a.dL_dcolor[cb + 2 * HW];
      if (a.dL_ddepth) dD = a.dL_ddepth[gp];
      if (a.dL_dalpha) dA = a.dL_dalpha[gp];
    }
  }
  if (threadIdx.x == 0) s_max = 0;
  __syncthreads();
  if (last) atomicMax(&s_max, last);
  __syncthreads();
  const int max_last = (int)s_max;
  const float bg_dot = __ldg(sd.bg + 0) * dC0 + __ldg(sd.bg + 1) * dC1 + __ldg(sd.bg + 2) * dC2;

  float T = T_final;
  float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, accd = 0.f;
  float last_a = 0.f, last0 = 0.f, last1 = 0.f, last2 = 0.f, lastd = 0.f;

  const int nb = (max_last + kBwdBatch - 1) / kBwdBatch;
  for (int b = nb - 1; b >= 0; --b) {
    const int base = b * kBwdBatch;
    const int cnt = min(kBwdBatch, max_last - base);
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      uint32_t i = lo + base + threadIdx.x;
      uint32_t g = a.sorted_gid[i];
      s_pidx[threadIdx.x] = a.sorted_pidx[i];
      float2 m = a.xy[g];
      float4 co = a.conic_op[g];
      s_xyt[threadIdx.x] = make_float4(m.x, m.y, alpha_threshold(co.w), 0.0f);
      s_co[threadIdx.x] = make_float4(-0.5f * co.x, -co.y, -0.5f * co.z, co.w);
      s_rgbd[threadIdx.x] = a.rgbd[g];
    }
    __syncthreads();
    uint32_t keep[kBwdBatch / 32];
#pragma unroll
    for (int r = 0; r < kBwdBatch / 32; ++r) {
      const int j = r * 32 + lane;
      bool k = false;
      if (j < cnt) {
        const float4 xyt = s_xyt[j];
        const float4 co = s_co[j];
        k = box_may_contribute(make_float2(xyt.x, xyt.y), co.x, co.y, co.z, xyt.z, bxf0, bxf1, byf0, byf1);
      }
      keep[r] = __ballot_sync(0xffffffffu, k);
      if (lane == 0) s_keep[warp][r] = keep[r];
    }
#pragma unroll
    for (int r = kBwdBatch / 32 - 1; r >= 0; --r) {
     uint32_t mk = keep[r];
     while (mk) {
      const int bit = 31 - __clz(mk);
      mk &= ~(1u << bit);
      const int j = r * 32 + bit;
      const int c = base + j;
      float v[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = 0.f;
      bool contrib = false;
      if (c < (int)last) {
        const float4 m = s_xyt[j];
        float4 co = s_co[j];
        float dx = m.x - pxf, dy = m.y - pyf;
        float power = gauss_power(co.x, co.y, co.z, dx, dy);
        if (!(power > 0.0f || power < m.z)) {
          float G = exp_ref_inrange(power);
          float alpha = fminf(CFGS_ALPHA_MAX, co.w * G);
          if (alpha >= CFGS_ALPHA_MIN) {
            contrib = true;
            float4 col = s_rgbd[j];
            float one_m = 1.0f - alpha;
            T = T / one_m;
            float w = alpha * T;
            v[6] = dC0 * w;
            v[7] = dC1 * w;
            v[8] = dC2 * w;
            v[9] = dD * w;
            acc0 = last_a * last0 + (1.f - last_a) * acc0;
            acc1 = last_a * last1 + (1.f - last_a) * acc1;
            acc2 = last_a * last2 + (1.f - last_a) * acc2;
            accd = last_a * lastd + (1.f - last_a) * accd;
            last0 = col.x;
            last1 = col.y;
            last2 = col.z;
            lastd = col.w;
            last_a = alpha;
            float dLda = (col.x - acc0) * dC0 + (col.y - acc1) * dC1 + (col.z - acc2) * dC2 +
                         (col.w - accd) * dD;
            dLda *= T;
            float tf = T_final / one_m;
            dLda += tf * (dA - bg_dot);
            v[5] = G * dLda;                 // d/d opacity (straight through the 0.99 clamp)
            float dLdp = G * (co.w * dLda);  // d/d power
            // power = ca dx^2 + cb dx dy + cc dy^2, dx = mean.x - pixel.x
            v[0] = dLdp * (2.f * co.x * dx + co.y * dy);
            v[1] = dLdp * (2.f * co.z * dy + co.y * dx);
            v[2] = -0.5f * dx * dx * dLdp;  // d/d conic.a
            v[3] = -dx * dy * dLdp;         // d/d conic.b
            v[4] = -0.5f * dy * dy * dLdp;  // d/d conic.c
          }
        }
      }
      if (__ballot_sync(0xffffffffu, contrib)) {
        float r = warp_transpose_reduce16(v, lane);
        int k = lane >> 1;
        if (!(lane & 1) && k < 10) s_part[warp][j][k] = r;
      } else if (lane < 10) {
        s_part[warp][j][lane] = 0.f;
      }
     }
    }
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const int j = threadIdx.x;
      float sum[10];
#pragma unroll
      for (int k = 0; k < 10; ++k) sum[k] = 0.f;
#pragma unroll
      for (int w = 0; w < kWarps; ++w)
        if ((s_keep[w][j >> 5] >> (j & 31)) & 1u)
#pragma unroll
          for (int k = 0; k < 10; ++k) sum[k] += s_part[w][j][k];
      float4* rec = a.records + (size_t)kRecordFloat4 * s_pidx[threadIdx.x];
      rec[0] = make_float4(sum[0], sum[1], sum[2], sum[3]);
      rec[1] = make_float4(sum[4], sum[5], sum[6], sum[7]);
      rec[2] = make_float4(sum[8], sum[9], 0.f, 0.f);
    }
  }
  for (int i = max_last + threadIdx.x; i < n; i += blockDim.x) {
    float4* rec = a.records + (size_t)kRecordFloat4 * a.sorted_pidx[lo + i];
    rec[0] = make_float4(0.f, 0.f, 0.f, 0.f);
    rec[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    rec[2] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// SH basis values b[k] and their partial derivatives along the unit direction.
__device__ __forceinline__ int sh_basis_grad(int deg, float x, float y, float z, float* b, float* bx, float* by,
                                             float* bz) {
  for (int k = 0; k < 16; ++k) b[k] = bx[k] = by[k] = bz[k] = 0.f;
  b[0] = CFGS_SH_C0;
  if (deg < 1) return 1;
  b[1] = -CFGS_SH_C1 * y; by[1] = -CFGS_SH_C1;
  b[2] = CFGS_SH_C1 * z;  bz[2] = CFGS_SH_C1;
  b[3] = -CFGS_SH_C1 * x; bx[3] = -CFGS_SH_C1;
  if (deg < 2) return 4;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  b[4] = CFGS_SH_C2_0 * xy; bx[4] = CFGS_SH_C2_0 * y; by[4] = CFGS_SH_C2_0 * x;
  b[5] = CFGS_SH_C2_1 * yz; by[5] = CFGS_SH_C2_1 * z; bz[5] = CFGS_SH_C2_1 * y;
  b[6] = CFGS_SH_C2_2 * (2.f * zz - xx - yy);
  bx[6] = -2.f * CFGS_SH_C2_2 * x; by[6] = -2.f * CFGS_SH_C2_2 * y; bz[6] = 4.f * CFGS_SH_C2_2 * z;
  b[7] = CFGS_SH_C2_3 * xz; bx[7] = CFGS_SH_C2_3 * z; bz[7] = CFGS_SH_C2_3 * x;
  b[8] = CFGS_SH_C2_4 * (xx - yy); bx[8] = 2.f * CFGS_SH_C2_4 * x; by[8] = -2.f * CFGS_SH_C2_4 * y;
  if (deg < 3) return 9;
  b[9] = CFGS_SH_C3_0 * y * (3.f * xx - yy);
  bx[9] = CFGS_SH_C3_0 * 6.f * xy; by[9] = CFGS_SH_C3_0 * (3.f * xx - 3.f * yy);
  b[10] = CFGS_SH_C3_1 * xy * z;
  bx[10] = CFGS_SH_C3_1 * yz; by[10] = CFGS_SH_C3_1 * xz; bz[10] = CFGS_SH_C3_1 * xy;
  b[11] = CFGS_SH_C3_2 * y * (4.f * zz - xx - yy);
  bx[11] = -2.f * CFGS_SH_C3_2 * xy; by[11] = CFGS_SH_C3_2 * (4.f * zz - xx - 3.f * yy);
  bz[11] = 8.f * CFGS_SH_C3_2 * yz;
  b[12] = CFGS_SH_C3_3 * z * (2.f * zz - 3.f * xx - 3.f * yy);
  bx[12] = -6.f * CFGS_SH_C3_3 * xz; by[12] = -6.f * CFGS_SH_C3_3 * yz;
  bz[12] = CFGS_SH_C3_3 * (6.f * zz - 3.f * xx - 3.f * yy);
  b[13] = CFGS_SH_C3_4 * x * (4.f * zz - xx - yy);
  bx[13] = CFGS_SH_C3_4 * (4.f * zz - 3.f * xx - yy); by[13] = -2.f * CFGS_SH_C3_4 * xy;
  bz[13] = 8.f * CFGS_SH_C3_4 * xz;
  b[14] = CFGS_SH_C3_5 * z * (xx - yy);
  bx[14] = 2.f * CFGS_SH_C3_5 * xz; by[14] = -2.f * CFGS_SH_C3_5 * yz; bz[14] = CFGS_SH_C3_5 * (xx - yy);
  b[15] = CFGS_SH_C3_6 * x * (xx - 3.f * yy);
  bx[15] = CFGS_SH_C3_6 * (3.f * xx - 3.f * yy); by[15] = -6.f * CFGS_SH_C3_6 * xy;
  return 16;
}

// Full form: all eight gradient arrays. Pose-only form (pose_partials set): only
// dL/dmean (through projection, covariance and SH view direction) is formed and the
// block's SE(3) gradient terms — sum g and sum (R p) x g in float64 with the scene's
// float64 rotation and the un-posed positions p — go to pose_partials[block].
template <class Scenes>
__global__ void __launch_bounds__(256) k_preprocess_bwd(PreBwdArgs<Scenes> a) {
  __shared__ double s_red[8][6];
  const SceneDesc& sd = a.scenes.for_block(blockIdx.x);
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool pose_only = a.pose_partials != nullptr;
  if (!pose_only && idx >= a.total_slots) return;
  if ((int64_t)a.counts->num_rendered > a.cap) return;  // forward overflowed: outputs untouched
  const bool valid = idx < a.total_slots && idx - sd.gauss_base < sd.num_gaussians;
  const int M = sd.sh_coeffs;
  const uint32_t nt = (valid && a.radii[idx] > 0) ? a.geom.touched[idx] : 0u;
  float dmean[3] = {0.f, 0.f, 0.f};
  if (nt == 0 && !pose_only) {
    for (int k = 0; k < 3; ++k) {
      a.out.dL_dmeans2D[3 * idx + k] = 0.f;
      a.out.dL_dcolors[3 * idx + k] = 0.f;
      a.out.dL_dmeans3D[3 * idx + k] = 0.f;
      if (a.out.dL_dscales) a.out.dL_dscales[3 * idx + k] = 0.f;
    }
    a.out.dL_dopacity[idx] = 0.f;
    for (int k = 0; k < 6; ++k) a.out.dL_dcov3D[6 * idx + k] = 0.f;
    if (a.out.dL_drotations)
      for (int k = 0; k < 4; ++k) a.out.dL_drotations[4 * idx + k] = 0.f;
    if (a.out.dL_dsh)
      for (int k = 0; k < 3 * M; ++k) a.out.dL_dsh[(size_t)idx * 3 * M + k] = 0.f;
    return;
  }
  if (nt > 0) {
    // ---- sum this Gaussian's per-tile records in pre-sort order ------------------
    float acc[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = 0.f;
    const float4* rec = a.records + (size_t)kRecordFloat4 * a.geom.offset[idx];
    for (uint32_t i = 0; i < nt; ++i) {
      float4 r0 = rec[3 * i + 0], r1 = rec[3 * i + 1], r2 = rec[3 * i + 2];
      acc[0] += r0.x; acc[1] += r0.y; acc[2] += r0.z; acc[3] += r0.w;
      acc[4] += r1.x; acc[5] += r1.y; acc[6] += r1.z; acc[7] += r1.w;
      acc[8] += r2.x; acc[9] += r2.y;
    }
    const float W = (float)sd.W, H = (float)sd.H;
    const float dndc_x = acc[0] * (0.5f * W), dndc_y = acc[1] * (0.5f * H);
    const float dcol[3] = {acc[6], acc[7], acc[8]};
    if (!pose_only) {
      a.out.dL_dmeans2D[3 * idx + 0] = dndc_x;
      a.out.dL_dmeans2D[3 * idx + 1] = dndc_y;
      a.out.dL_dmeans2D[3 * idx + 2] = 0.f;
      a.out.dL_dopacity[idx] = acc[5];
      a.out.dL_dcolors[3 * idx + 0] = dcol[0];
      a.out.dL_dcolors[3 * idx + 1] = dcol[1];
      a.out.dL_dcolors[3 * idx + 2] = dcol[2];
    }

    float V[16], P[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) V[i] = __ldg(sd.V + i);
#pragma unroll
    for (int i = 0; i < 16; ++i) P[i] = __ldg(sd.P + i);
    const float3 pm = posed_mean(sd, a.g.means3D, (size_t)idx);
    const float px = pm.x, py = pm.y, pz = pm.z;

    // ---- recompute view-space centre and the 2D covariance pieces ----------------
    float t[3];
    for (int i = 0; i < 3; ++i) t[i] = V[i] * px + V[4 + i] * py + V[8 + i] * pz + V[12 + i];
    float cov[6];
    float sx = 0, sy = 0, sz = 0, qr = 0, qx = 0, qy = 0, qz = 0, R[9];
    const float mod = sd.scale_modifier;
    if (a.g.cov3D_precomp) {
      for (int k = 0; k < 6; ++k) cov[k] = a.g.cov3D_precomp[6 * idx + k];
    } else {
      sx = mod * a.g.scales[3 * idx + 0];
      sy = mod * a.g.scales[3 * idx + 1];
      sz = mod * a.g.scales[3 * idx + 2];
      qr = a.g.rotations[4 * idx + 0];
      qx = a.g.rotations[4 * idx + 1];
      qy = a.g.rotations[4 * idx + 2];
      qz = a.g.rotations[4 * idx + 3];
      R[0] = 1.f - 2.f * (qy * qy + qz * qz);
      R[1] = 2.f * (qx * qy - qr * qz);
      R[2] = 2.f * (qx * qz + qr * qy);
      R[3] = 2.f * (qx * qy + qr * qz);
      R[4] = 1.f - 2.f * (qx * qx + qz * qz);
      R[5] = 2.f * (qy * qz - qr * qx);
      R[6] = 2.f * (qx * qz - qr * qy);
      R[7] = 2.f * (qy * qz + qr * qx);
      R[8] = 1.f - 2.f * (qx * qx + qy * qy);
      const float s3[3] = {sx, sy, sz};
      float Mm[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Mm[3 * i + j] = R[3 * i + j] * s3[j];
      const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
      for (int k = 0; k < 6; ++k) {
        const float* u = Mm + 3 * ii[k];
        const float* w = Mm + 3 * jj[k];
        cov[k] = u[0] * w[0] + u[1] * w[1] + u[2] * w[2];
      }
    }
    const float limx = 1.3f * sd.tanfovx, limy = 1.3f * sd.tanfovy;
    const float txtz = t[0] / t[2], tytz = t[1] / t[2];
    const float tx = fminf(limx, fmaxf(-limx, txtz)) * t[2];
    const float ty = fminf(limy, fmaxf(-limy, tytz)) * t[2];
    const float xmask = (txtz < -limx || txtz > limx) ? 0.f : 1.f;
    const float ymask = (tytz < -limy || tytz > limy) ? 0.f : 1.f;
    const float tz = t[2], tz2 = tz * tz, tz3 = tz2 * tz;
    const float fx = sd.focal_x, fy = sd.focal_y;
    const float J00 = fx / tz, J02 = -(fx * tx) / tz2, J11 = fy / tz, J12 = -(fy * ty) / tz2;
    float T0[3], T1[3];
    for (int j = 0; j < 3; ++j) {
      T0[j] = J00 * V[4 * j + 0] + J02 * V[4 * j + 2];
      T1[j] = J11 * V[4 * j + 1] + J12 * V[4 * j + 2];
    }
    const float S[9] = {cov[0], cov[1], cov[2], cov[1], cov[3], cov[4], cov[2], cov[4], cov[5]};
    float u[3], v[3];
    for (int i = 0; i < 3; ++i) {
      u[i] = S[3 * i] * T0[0] + S[3 * i + 1] * T0[1] + S[3 * i + 2] * T0[2];
      v[i] = S[3 * i] * T1[0] + S[3 * i + 1] * T1[1] + S[3 * i + 2] * T1[2];
    }
    const float ca = T0[0] * u[0] + T0[1] * u[1] + T0[2] * u[2] + 0.3f;
    const float cb = T0[0] * v[0] + T0[1] * v[1] + T0[2] * v[2];
    const float cc = T1[0] * v[0] + T1[1] * v[1] + T1[2] * v[2] + 0.3f;

    // ---- conic (A,B,C) -> 2D covariance (a,b,c) -----------------------------------
    const float dA = acc[2], dB = acc[3], dC = acc[4];
    const float det = ca * cc - cb * cb;
    const float id = 1.f / det, id2 = id * id;
    const float da = dA * (-cc * cc * id2) + dB * (cb * cc * id2) + dC * (id - ca * cc * id2);
    const float db = dA * (2.f * cb * cc * id2) + dB * (-id - 2.f * cb * cb * id2) + dC * (2.f * ca * cb * id2);
    const float dc = dA * (id - ca * cc * id2) + dB * (ca * cb * id2) + dC * (-ca * ca * id2);

    // ---- 2D covariance -> 3D covariance and the rows of T = J W ------------------
    float dcov[6];
    dcov[0] = da * T0[0] * T0[0] + db * T0[0] * T1[0] + dc * T1[0] * T1[0];
    dcov[3] = da * T0[1] * T0[1] + db * T0[1] * T1[1] + dc * T1[1] * T1[1];
    dcov[5] = da * T0[2] * T0[2] + db * T0[2] * T1[2] + dc * T1[2] * T1[2];
    dcov[1] = 2.f * da * T0[0] * T0[1] + db * (T0[0] * T1[1] + T0[1] * T1[0]) + 2.f * dc * T1[0] * T1[1];
    dcov[2] = 2.f * da * T0[0] * T0[2] + db * (T0[0] * T1[2] + T0[2] * T1[0]) + 2.f * dc * T1[0] * T1[2];
    dcov[4] = 2.f * da * T0[1] * T0[2] + db * (T0[1] * T1[2] + T0[2] * T1[1]) + 2.f * dc * T1[1] * T1[2];
    if (!pose_only)
      for (int k = 0; k < 6; ++k) a.out.dL_dcov3D[6 * idx + k] = dcov[k];
    float dT0[3], dT1[3];
    for (int i = 0; i < 3; ++i) {
      dT0[i] = 2.f * da * u[i] + db * v[i];
      dT1[i] = db * u[i] + 2.f * dc * v[i];
    }
    float dJ00 = 0, dJ02 = 0, dJ11 = 0, dJ12 = 0;
    for (int j = 0; j < 3; ++j) {
      dJ00 += dT0[j] * V[4 * j + 0];
      dJ02 += dT0[j] * V[4 * j + 2];
      dJ11 += dT1[j] * V[4 * j + 1];
      dJ12 += dT1[j] * V[4 * j + 2];
    }
    float dt[3];
    dt[0] = xmask * (dJ02 * (-fx / tz2));
    dt[1] = ymask * (dJ12 * (-fy / tz2));
    dt[2] = dJ00 * (-fx / tz2) + dJ11 * (-fy / tz2) + dJ02 * (2.f * fx * tx / tz3) +
            dJ12 * (2.f * fy * ty / tz3) + acc[9];  // + d/d depth (depth = view z)
    for (int j = 0; j < 3; ++j) dmean[j] = V[4 * j + 0] * dt[0] + V[4 * j + 1] * dt[1] + V[4 * j + 2] * dt[2];

    // ---- projection: NDC = hom.xy / (hom.w + 1e-7) -------------------------------
    {
      const float hx = P[0] * px + P[4] * py + P[8] * pz + P[12];
      const float hy = P[1] * px + P[5] * py + P[9] * pz + P[13];
      const float hw = P[3] * px + P[7] * py + P[11] * pz + P[15];
      const float wi = 1.f / (hw + 0.0000001f);
      const float wi2 = wi * wi;
      for (int j = 0; j < 3; ++j) {
        dmean[j] += dndc_x * (P[4 * j + 0] * wi - hx * wi2 * P[4 * j + 3]) +
                    dndc_y * (P[4 * j + 1] * wi - hy * wi2 * P[4 * j + 3]);
      }
    }

    // ---- SH colour ----------------------------------------------------------------
    if (a.g.shs) {
      const uint8_t cl = a.geom.clamped[idx];
      const float g0 = (cl & 1) ? 0.f : dcol[0];
      const float g1 = (cl & 2) ? 0.f : dcol[1];
      const float g2 = (cl & 4) ? 0.f : dcol[2];
      const float* sh = a.g.shs + (size_t)idx * 3 * M;
      float* dsh = (!pose_only && a.out.dL_dsh) ? a.out.dL_dsh + (size_t)idx * 3 * M : nullptr;
      const float cx = __ldg(sd.campos + 0), cy = __ldg(sd.campos + 1), cz = __ldg(sd.campos + 2);
      const float ddx = px - cx, ddy = py - cy, ddz = pz - cz;
      const float len = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
      const float x = ddx / len, y = ddy / len, z = ddz / len;
      float b[16], bx[16], by[16], bz[16];
      const int nb = sh_basis_grad(sd.sh_degree, x, y, z, b, bx, by, bz);
      float gdx = 0.f, gdy = 0.f, gdz = 0.f;
      for (int k = 0; k < M; ++k) {
        if (k < nb) {
          if (dsh) {
            dsh[3 * k + 0] = b[k] * g0;
            dsh[3 * k + 1] = b[k] * g1;
            dsh[3 * k + 2] = b[k] * g2;
          }
          const float s = sh[3 * k] * g0 + sh[3 * k + 1] * g1 + sh[3 * k + 2] * g2;
          gdx += s * bx[k];
          gdy += s * by[k];
          gdz += s * bz[k];
        } else if (dsh) {
          dsh[3 * k + 0] = 0.f;
          dsh[3 * k + 1] = 0.f;
          dsh[3 * k + 2] = 0.f;
        }
      }
      // d/d(unnormalised direction) = (g - dir (dir . g)) / |d|
      const float dotv = x * gdx + y * gdy + z * gdz;
      dmean[0] += (gdx - x * dotv) / len;
      dmean[1] += (gdy - y * dotv) / len;
      dmean[2] += (gdz - z * dotv) / len;
    }
    if (!pose_only) {
      for (int j = 0; j < 3; ++j) a.out.dL_dmeans3D[3 * idx + j] = dmean[j];

      // ---- 3D covariance -> scale and rotation ----------------------------------
      if (!a.g.cov3D_precomp) {
        const float s3[3] = {sx, sy, sz};
        float Mm[9];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Mm[3 * i + j] = R[3 * i + j] * s3[j];
        // symmetric matrix-entry derivative: diagonal = dcov, off-diagonal = dcov / 2
        const float G[9] = {dcov[0], 0.5f * dcov[1], 0.5f * dcov[2], 0.5f * dcov[1], dcov[3],
                            0.5f * dcov[4], 0.5f * dcov[2], 0.5f * dcov[4], dcov[5]};
        float dM[9];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            dM[3 * i + j] = 2.f * (G[3 * i] * Mm[j] + G[3 * i + 1] * Mm[3 + j] + G[3 * i + 2] * Mm[6 + j]);
        float dR[9];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) dR[3 * i + j] = dM[3 * i + j] * s3[j];
        for (int j = 0; j < 3; ++j) {
          const float ds = dM[j] * R[j] + dM[3 + j] * R[3 + j] + dM[6 + j] * R[6 + j];
          a.out.dL_dscales[3 * idx + j] = ds * mod;
        }
        const float r = qr, x = qx, y = qy, z = qz;
        const float dr = 2.f * (-z * dR[1] + y * dR[2] + z * dR[3] - x * dR[5] - y * dR[6] + x * dR[7]);
        const float dxq = 2.f * (y * dR[1] + z * dR[2] + y * dR[3] - 2.f * x * dR[4] - r * dR[5] + z * dR[6] +
                                 r * dR[7] - 2.f * x * dR[8]);
        const float dyq = 2.f * (-2.f * y * dR[0] + x * dR[1] + r * dR[2] + x * dR[3] + z * dR[5] - r * dR[6] +
                                 z * dR[7] - 2.f * y * dR[8]);
        const float dzq = 2.f * (-2.f * z * dR[0] - r * dR[1] + x * dR[2] + r * dR[3] - 2.f * z * dR[4] +
                                 y * dR[5] + x * dR[6] + y * dR[7]);
        a.out.dL_drotations[4 * idx + 0] = dr;
        a.out.dL_drotations[4 * idx + 1] = dxq;
        a.out.dL_drotations[4 * idx + 2] = dyq;
        a.out.dL_drotations[4 * idx + 3] = dzq;
      }
      return;
    }
  }
  if (!pose_only) return;
  // ---- pose-only form: the block's SE(3) gradient terms in float64 -----------------
  double term[6] = {0, 0, 0, 0, 0, 0};
  if (nt > 0 && sd.pose) {
    const double* R64 = sd.pose->R64;
    const double p0 = a.g.means3D[3 * idx], p1 = a.g.means3D[3 * idx + 1], p2 = a.g.means3D[3 * idx + 2];
    const double g0 = dmean[0], g1 = dmean[1], g2 = dmean[2];
    const double q0 = R64[0] * p0 + R64[1] * p1 + R64[2] * p2;
    const double q1 = R64[3] * p0 + R64[4] * p1 + R64[5] * p2;
    const double q2 = R64[6] * p0 + R64[7] * p1 + R64[8] * p2;
    term[0] = g0;
    term[1] = g1;
    term[2] = g2;
    term[3] = q1 * g2 - q2 * g1;
    term[4] = q2 * g0 - q0 * g2;
    term[5] = q0 * g1 - q1 * g0;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double v = term[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += s_red[w][threadIdx.x];
    a.pose_partials[(size_t)blockIdx.x * 9 + threadIdx.x] = v;
  } else if (threadIdx.x < 9) {
    a.pose_partials[(size_t)blockIdx.x * 9 + threadIdx.x] = 0.0;
  }
}

template <class Scenes>
void launch_render_bwd(const RenderBwdArgs<Scenes>& a, int tiles, cudaStream_t st) {
  k_render_bwd<Scenes><<<tiles, kTilePixels, 0, st>>>(a);
}
template <class Scenes>
void launch_preprocess_bwd(const PreBwdArgs<Scenes>& a, int blocks, cudaStream_t st) {
  k_preprocess_bwd<Scenes><<<blocks, 256, 0, st>>>(a);
}
template void launch_render_bwd<SingleScene>(const RenderBwdArgs<SingleScene>&, int, cudaStream_t);
template void launch_render_bwd<SceneTable>(const RenderBwdArgs<SceneTable>&, int, cudaStream_t);
template void launch_preprocess_bwd<SingleScene>(const PreBwdArgs<SingleScene>&, int, cudaStream_t);
template void launch_preprocess_bwd<SceneTable>(const PreBwdArgs<SceneTable>&, int, cudaStream_t);

}  // namespace cfgs

using namespace cfgs;

extern "C" int cfgs_render_backward(const CfgsSettings* s, int32_t num_gaussians, const void* geom, const void* image,
                                    const void* binning, int64_t capacity, void* scratch, const float* dL_dcolor,
                                    const float* dL_ddepth, const float* dL_dalpha, void* stream) {
  if (!s || !geom || !image || !binning || !scratch || !dL_dcolor || !s->bg || num_gaussians < 0)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (s->image_width <= 0 || s->image_height <= 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity < 0 || capacity > 0x7fffffffll) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  ImageLayout IL(s->image_width, s->image_height);
  ImageView iv(const_cast<void*>(image), s->image_width, s->image_height);
  GeomView gv(const_cast<void*>(geom), num_gaussians);
  BinningView bv(const_cast<void*>(binning), capacity);
  RenderBwdArgs<SingleScene> ra;
  ra.scenes.d = single_scene_desc(s, num_gaussians, 0);
  ra.tile_range = iv.tile_range;
  ra.sorted_gid = bv.sorted_gid;
  ra.sorted_pidx = bv.sorted_pidx;
  ra.xy = gv.xy;
  ra.conic_op = gv.conic_op;
  ra.rgbd = gv.rgbd;
  ra.final_T = iv.final_T;
  ra.n_contrib = iv.n_contrib;
  ra.dL_dcolor = dL_dcolor;
  ra.dL_ddepth = dL_ddepth;
  ra.dL_dalpha = dL_dalpha;
  ra.color = nullptr;
  ra.target = nullptr;
  ra.records = static_cast<float4*>(scratch);
  ra.cap = capacity;
  ra.counts = iv.counts;
  launch_render_bwd(ra, IL.num_tiles, st);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_preprocess_backward(const CfgsSettings* s, const CfgsGaussians* g, const int32_t* radii,
                                        const void* geom, const void* image, int64_t capacity, const void* scratch,
                                        const CfgsGradients* out, void* stream) {
  if (!s || !g || !geom || !image || !scratch || !out || !s->viewmatrix || !s->projmatrix)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (g->num_gaussians == 0) return CFGS_OK;
  if (g->num_gaussians < 0 || !radii || !g->means3D || !g->opacities) return CFGS_ERR_INVALID_ARGUMENT;
  if (!out->dL_dmeans2D || !out->dL_dcolors || !out->dL_dopacity || !out->dL_dmeans3D || !out->dL_dcov3D)
    return CFGS_ERR_INVALID_ARGUMENT;
  if (!g->cov3D_precomp && (!out->dL_dscales || !out->dL_drotations || !g->scales || !g->rotations))
    return CFGS_ERR_INVALID_ARGUMENT;
  if ((g->shs == nullptr) == (g->colors_precomp == nullptr)) return CFGS_ERR_INVALID_ARGUMENT;
  if (g->shs && !s->campos) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity < 0 || capacity > 0x7fffffffll) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  ImageView iv(const_cast<void*>(image), s->image_width, s->image_height);
  PreBwdArgs<SingleScene> pa;
  pa.scenes.d = single_scene_desc(s, g->num_gaussians, g->sh_coeffs);
  pa.g = *g;
  pa.radii = radii;
  pa.geom = GeomView(const_cast<void*>(geom), g->num_gaussians);
  pa.records = static_cast<const float4*>(scratch);
  pa.out = *out;
  pa.total_slots = g->num_gaussians;
  pa.cap = capacity;
  pa.counts = iv.counts;
  pa.pose_partials = nullptr;
  launch_preprocess_bwd(pa, div_up(g->num_gaussians, 256), st);
  CFGS_CHECK_LAUNCH(s->debug, st);
  return CFGS_OK;
}

extern "C" int cfgs_backward(const CfgsSettings* s, const CfgsGaussians* g, const int32_t* radii, const void* geom,
                             const void* image, const void* binning, int64_t capacity, void* scratch,
                             const float* dL_dcolor, const float* dL_ddepth, const float* dL_dalpha,
                             const CfgsGradients* out, void* stream) {
  if (!g) return CFGS_ERR_INVALID_ARGUMENT;
  if (g->num_gaussians == 0) return CFGS_OK;
  int st = cfgs_render_backward(s, g->num_gaussians, geom, image, binning, capacity, scratch, dL_dcolor, dL_ddepth,
                                dL_dalpha, stream);
  if (st != CFGS_OK) return st;
  return cfgs_preprocess_backward(s, g, radii, geom, image, capacity, scratch, out, stream);
}

// ---- allocation-free backward ----------------------------------------------------
// Some callers cannot allocate device memory when they call the rasteriser: plugin
// hosts that hand a plugin only its input and output buffers, and services that must
// not allocate once they are serving. This entry point runs the same two kernels as
// cfgs_backward, but the per-instance gradient records live in the fixed array below
// instead of a caller-provided scratch buffer. Every GPU that loads this library holds
// the array (30 MiB) until the process exits.
static __device__ __align__(256) float4 g_noalloc_records[(size_t)CFGS_NOALLOC_MAX_INSTANCES * kRecordFloat4];

namespace {
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kNoallocMaxDevices] = {};

// Device address of g_noalloc_records on the current device. The host-side name of
// the array is only a stand-in, so the address is looked up once per device, with
// that device current, and cached.
int noalloc_records(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoallocMaxDevices) return CFGS_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_records) != cudaSuccess || p == nullptr) return CFGS_ERR_LAUNCH;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return CFGS_OK;
}
}  // namespace

extern "C" int cfgs_backward_noalloc(const CfgsSettings* s, const CfgsGaussians* g, const int32_t* radii,
                                     const void* geom, const void* image, const void* binning, int64_t capacity,
                                     const float* dL_dcolor, const float* dL_ddepth, const float* dL_dalpha,
                                     const CfgsGradients* out, void* stream) {
  if (capacity < 0) return CFGS_ERR_INVALID_ARGUMENT;
  if (capacity > CFGS_NOALLOC_MAX_INSTANCES) return CFGS_ERR_TOO_LARGE;
  void* records = nullptr;
  int st = noalloc_records(&records);
  if (st != CFGS_OK) return st;
  return cfgs_backward(s, g, radii, geom, image, binning, capacity, records, dL_dcolor, dL_ddepth, dL_dalpha, out,
                       stream);
}
