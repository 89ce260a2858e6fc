// Backward, part 2: the per-Gaussian preprocess backward (conic -> 2D covariance ->
// 3D covariance -> scale/rotation, projection -> mean, SH -> coefficients and view
// direction), in a full form (all eight gradient arrays, the drop-in path) and a
// pose-only form (dL/dmean reduced straight into SE(3) gradient terms, batched solves).
//
// Phase 1 sums each Gaussian's per-tile records (contiguous: instance indices
// [offset, offset + touched)) eight lanes per Gaussian, four Gaussians per warp at a
// time: strided 48-byte record loads of the records the render backward wrote (one byte
// per instance says which), a transposing reduction inside each group of eight lanes,
// the sums to shared memory. Phase 2 is one thread per Gaussian. Both
// orders are fixed, so the result is deterministic.
#include "cfgs_internal.cuh"
#include "kernels.cuh"

namespace cfgs {

// Sums 16 per-lane values over each group of eight lanes (lanes 8m .. 8m+7) in 14
// shuffles; lane 8m + s ends with the group totals of value indices 2s and 2s + 1 in
// v[0] and v[1].
__device__ __forceinline__ void group8_sum16(float (&v)[16], int lane) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const bool up = lane & 4;
    const float send = up ? v[k] : v[k + 8];
    const float keep = up ? v[k + 8] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const bool up = lane & 2;
    const float send = up ? v[k] : v[k + 4];
    const float keep = up ? v[k + 4] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool up = lane & 1;
    const float send = up ? v[k] : v[k + 2];
    const float keep = up ? v[k + 2] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
  }
}

// SH backward at unit direction (x,y,z): dL/dsh[k][c] = b_k g_c (g already masked by
// the forward's clamp) and the gradient of sum_k (sh_k . g) b_k with respect to the
// direction. The basis follows utils/sh_utils.py:57-112.
__device__ __forceinline__ void sh_backward(int deg, int M, const float* sh, float g0, float g1, float g2, float x,
                                            float y, float z, float* dsh, float& gdx, float& gdy, float& gdz) {
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  float b[16];
  b[0] = CFGS_SH_C0;
  b[1] = -CFGS_SH_C1 * y;
  b[2] = CFGS_SH_C1 * z;
  b[3] = -CFGS_SH_C1 * x;
  b[4] = CFGS_SH_C2_0 * xy;
  b[5] = CFGS_SH_C2_1 * yz;
  b[6] = CFGS_SH_C2_2 * (2.f * zz - xx - yy);
  b[7] = CFGS_SH_C2_3 * xz;
  b[8] = CFGS_SH_C2_4 * (xx - yy);
  b[9] = CFGS_SH_C3_0 * y * (3.f * xx - yy);
  b[10] = CFGS_SH_C3_1 * xy * z;
  b[11] = CFGS_SH_C3_2 * y * (4.f * zz - xx - yy);
  b[12] = CFGS_SH_C3_3 * z * (2.f * zz - 3.f * xx - 3.f * yy);
  b[13] = CFGS_SH_C3_4 * x * (4.f * zz - xx - yy);
  b[14] = CFGS_SH_C3_5 * z * (xx - yy);
  b[15] = CFGS_SH_C3_6 * x * (xx - 3.f * yy);
  const int nb = (deg + 1) * (deg + 1);
#pragma unroll
  for (int k = 1; k < 16; ++k)
    if (k >= nb) b[k] = 0.f;
  // s_k = sh_k . g for every coefficient k (12 vector loads when aligned)
  float sk[16];
  if (M == 16 && (((uintptr_t)sh) & 15) == 0) {
    const float4* s4 = reinterpret_cast<const float4*>(sh);
    const float gc[3] = {g0, g1, g2};
#pragma unroll
    for (int k = 0; k < 16; ++k) sk[k] = 0.f;
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      const float4 f = s4[q];
      const float e[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = 4 * q + u;  // coefficient i / 3, channel i % 3
        sk[i / 3] = (i % 3 == 0) ? e[u] * gc[0] : sk[i / 3] + e[u] * gc[i % 3];
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < 16; ++k) sk[k] = k < nb ? sh[3 * k] * g0 + sh[3 * k + 1] * g1 + sh[3 * k + 2] * g2 : 0.f;
  }
#define CFGS_SK(k) sk[k]
  gdx = gdy = gdz = 0.f;
  if (deg > 0) {
    const float s1 = CFGS_SK(1), s2 = CFGS_SK(2), s3 = CFGS_SK(3);
    gdy -= CFGS_SH_C1 * s1;
    gdz += CFGS_SH_C1 * s2;
    gdx -= CFGS_SH_C1 * s3;
  }
  if (deg > 1) {
    const float s4 = CFGS_SK(4), s5 = CFGS_SK(5), s6 = CFGS_SK(6), s7 = CFGS_SK(7), s8 = CFGS_SK(8);
    gdx += CFGS_SH_C2_0 * y * s4 - 2.f * CFGS_SH_C2_2 * x * s6 + CFGS_SH_C2_3 * z * s7 + 2.f * CFGS_SH_C2_4 * x * s8;
    gdy += CFGS_SH_C2_0 * x * s4 + CFGS_SH_C2_1 * z * s5 - 2.f * CFGS_SH_C2_2 * y * s6 - 2.f * CFGS_SH_C2_4 * y * s8;
    gdz += CFGS_SH_C2_1 * y * s5 + 4.f * CFGS_SH_C2_2 * z * s6 + CFGS_SH_C2_3 * x * s7;
  }
  if (deg > 2) {
    const float s9 = CFGS_SK(9), s10 = CFGS_SK(10), s11 = CFGS_SK(11), s12 = CFGS_SK(12), s13 = CFGS_SK(13),
                s14 = CFGS_SK(14), s15 = CFGS_SK(15);
    gdx += CFGS_SH_C3_0 * 6.f * xy * s9 + CFGS_SH_C3_1 * yz * s10 - 2.f * CFGS_SH_C3_2 * xy * s11 -
           6.f * CFGS_SH_C3_3 * xz * s12 + CFGS_SH_C3_4 * (4.f * zz - 3.f * xx - yy) * s13 +
           2.f * CFGS_SH_C3_5 * xz * s14 + CFGS_SH_C3_6 * (3.f * xx - 3.f * yy) * s15;
    gdy += CFGS_SH_C3_0 * (3.f * xx - 3.f * yy) * s9 + CFGS_SH_C3_1 * xz * s10 +
           CFGS_SH_C3_2 * (4.f * zz - xx - 3.f * yy) * s11 - 6.f * CFGS_SH_C3_3 * yz * s12 -
           2.f * CFGS_SH_C3_4 * xy * s13 - 2.f * CFGS_SH_C3_5 * yz * s14 - 6.f * CFGS_SH_C3_6 * xy * s15;
    gdz += CFGS_SH_C3_1 * xy * s10 + 8.f * CFGS_SH_C3_2 * yz * s11 + CFGS_SH_C3_3 * (6.f * zz - 3.f * xx - 3.f * yy) * s12 +
           8.f * CFGS_SH_C3_4 * xz * s13 + CFGS_SH_C3_5 * (xx - yy) * s14;
  }
#undef CFGS_SK
  if (!dsh) return;
  const float gc[3] = {g0, g1, g2};
  if (M == 16 && (((uintptr_t)dsh) & 15) == 0) {
    float4* d4 = reinterpret_cast<float4*>(dsh);
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      float e[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) e[u] = b[(4 * q + u) / 3] * gc[(4 * q + u) % 3];
      d4[q] = make_float4(e[0], e[1], e[2], e[3]);
    }
  } else {
    for (int k = 0; k < M; ++k) {
      const float bk = k < 16 ? b[k] : 0.f;
      dsh[3 * k + 0] = bk * g0;
      dsh[3 * k + 1] = bk * g1;
      dsh[3 * k + 2] = bk * g2;
    }
  }
}

// The per-Gaussian part of the backward (one thread per Gaussian): record sums acc ->
// 2D grads, conic -> 2D covariance -> 3D covariance -> scale/rotation, projection ->
// mean, SH -> coefficients and view direction. SH coefficients are read from sh_src and
// their gradients written to dsh_dst (NULL: not wanted). Returns dL/dmean in dmean.
template <class Scenes>
__device__ __forceinline__ void gaussian_backward(const PreBwdArgs<Scenes>& a, const SceneDesc& sd, int64_t idx,
                                                  uint32_t nt, const float (&acc)[10], const float* sh_src,
                                                  float* dsh_dst, bool pose_only, float (&dmean)[3]) {
  const int M = sd.sh_coeffs;
  {
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
      const float4 q4 = (((uintptr_t)a.g.rotations) & 15) == 0
                            ? reinterpret_cast<const float4*>(a.g.rotations)[idx]
                            : make_float4(a.g.rotations[4 * idx], a.g.rotations[4 * idx + 1],
                                          a.g.rotations[4 * idx + 2], a.g.rotations[4 * idx + 3]);
      qr = q4.x;
      qx = q4.y;
      qy = q4.z;
      qz = q4.w;
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
    // With A = c/det, B = -b/det, C = a/det: dC/da = dA/dc = 1/det - ac/det^2, which is
    // -b^2/det^2 exactly; written that way it carries no cancellation (near-isotropic
    // conics, b ~ 0, would otherwise lose the term to the rounding of 1/det).
    const float dA = acc[2], dB = acc[3], dC = acc[4];
    const float det = ca * cc - cb * cb;
    const float id = 1.f / det, id2 = id * id;
    const float da = dA * (-cc * cc * id2) + dB * (cb * cc * id2) + dC * (-(cb * cb) * id2);
    const float db = dA * (2.f * cb * cc * id2) + dB * (-id - 2.f * cb * cb * id2) + dC * (2.f * ca * cb * id2);
    const float dc = dA * (-(cb * cb) * id2) + dB * (ca * cb * id2) + dC * (-ca * ca * id2);

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
      const float cx = __ldg(sd.campos + 0), cy = __ldg(sd.campos + 1), cz = __ldg(sd.campos + 2);
      const float ddx = px - cx, ddy = py - cy, ddz = pz - cz;
      const float len = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
      const float x = ddx / len, y = ddy / len, z = ddz / len;
      float gdx, gdy, gdz;
      sh_backward(sd.sh_degree, M, sh_src, g0, g1, g2, x, y, z, dsh_dst, gdx, gdy, gdz);
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
        float4 dq;
        dq.x = 2.f * (-z * dR[1] + y * dR[2] + z * dR[3] - x * dR[5] - y * dR[6] + x * dR[7]);
        dq.y = 2.f * (y * dR[1] + z * dR[2] + y * dR[3] - 2.f * x * dR[4] - r * dR[5] + z * dR[6] + r * dR[7] -
                      2.f * x * dR[8]);
        dq.z = 2.f * (-2.f * y * dR[0] + x * dR[1] + r * dR[2] + x * dR[3] + z * dR[5] - r * dR[6] + z * dR[7] -
                      2.f * y * dR[8]);
        dq.w = 2.f * (-2.f * z * dR[0] - r * dR[1] + x * dR[2] + r * dR[3] - 2.f * z * dR[4] + y * dR[5] +
                      x * dR[6] + y * dR[7]);
        if ((((uintptr_t)a.out.dL_drotations) & 15) == 0) {
          reinterpret_cast<float4*>(a.out.dL_drotations)[idx] = dq;
        } else {
          a.out.dL_drotations[4 * idx + 0] = dq.x;
          a.out.dL_drotations[4 * idx + 1] = dq.y;
          a.out.dL_drotations[4 * idx + 2] = dq.z;
          a.out.dL_drotations[4 * idx + 3] = dq.w;
        }
      }
    }
  }
}

// Zero gradients of a Gaussian that touched no tile (full form).
template <class Scenes>
__device__ __forceinline__ void zero_gradients(const PreBwdArgs<Scenes>& a, int64_t idx, int M, float* dsh_dst) {
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
  if (dsh_dst)
    for (int k = 0; k < 3 * M; ++k) dsh_dst[k] = 0.f;
}

// Full form: all eight gradient arrays. Pose-only form (pose_partials set): only
// dL/dmean (through projection, covariance and SH view direction) is formed and the
// block's SE(3) gradient terms — sum g and sum (R p) x g in float64 with the scene's
// float64 rotation and the un-posed positions p — go to pose_partials[block].
// With sh_bulk (degree-3 SH, 16-byte aligned), the block's 256 x 192 bytes of SH
// coefficients arrive in shared memory by one bulk copy issued before phase 1, and
// their gradients leave by one bulk store.
template <class Scenes, bool POSE>
__global__ void __launch_bounds__(256, POSE ? 4 : 3) k_preprocess_bwd(PreBwdArgs<Scenes> a) {
  extern __shared__ __align__(128) float4 s_sh[];  // [256][12] with sh_bulk
  __shared__ float s_acc[256][11];
  __shared__ double s_red[8][6];
  __shared__ __align__(8) uint64_t s_bar;
  if ((int64_t)a.counts->num_rendered > a.cap) return;  // forward overflowed: outputs untouched
  const SceneDesc& sd = a.scenes.for_block(blockIdx.x);
  constexpr bool pose_only = POSE;  // a.pose_partials is set exactly for this form
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t blk0 = (int64_t)blockIdx.x * blockDim.x;
  const int M = sd.sh_coeffs;
  const bool bulk = a.sh_bulk && a.g.shs != nullptr && M == kMaxShCoeffs;
  const uint32_t in_block = (uint32_t)min((int64_t)blockDim.x, a.total_slots - blk0);
  const uint32_t sh_bytes = in_block * 3u * kMaxShCoeffs * (uint32_t)sizeof(float);
  const uint32_t bar = smem_addr(&s_bar);
  if (bulk) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(sh_bytes) : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_addr(s_sh)),
                   "l"(a.g.shs + (size_t)blk0 * 3 * kMaxShCoeffs), "r"(sh_bytes), "r"(bar)
                   : "memory");
    }
  }

  // ---- phase 1: record sums, eight lanes per Gaussian ------------------------------
  {
    const int64_t gl = blk0 + warp * 32 + lane;  // this lane's Gaussian (metadata only)
    uint32_t nt_l = 0, off_l = 0;
    if (gl < a.total_slots && gl - sd.gauss_base < sd.num_gaussians && a.radii[gl] > 0) {
      nt_l = a.geom.touched[gl];
      off_l = a.geom.offset[gl];
    }
    const int sub = lane & 7, grp = lane >> 3;
    // The written marks of this lane's first two instance slots (sub, sub + 8) of all
    // eight rounds first: sixteen independent byte loads in flight together, so each
    // round below waits for its records only.
    uint32_t marks = 0;  // bits 2q, 2q + 1: round q's slots sub, sub + 8
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int src = 4 * q + grp;
      const uint32_t nt = __shfl_sync(0xffffffffu, nt_l, src);
      const uint32_t off = __shfl_sync(0xffffffffu, off_l, src);
      if ((uint32_t)sub < nt && __ldg(a.written + off + sub)) marks |= 1u << (2 * q);
      if ((uint32_t)sub + 8 < nt && __ldg(a.written + off + sub + 8)) marks |= 2u << (2 * q);
    }
    auto add_record = [&](float (&v)[16], uint32_t i) {
      const float4* rec = a.records + (size_t)kRecordFloat4 * i;
      const float4 r0 = rec[0], r1 = rec[1], r2 = rec[2];
      v[0] += r0.x; v[1] += r0.y; v[2] += r0.z; v[3] += r0.w;
      v[4] += r1.x; v[5] += r1.y; v[6] += r1.z; v[7] += r1.w;
      v[8] += r2.x; v[9] += r2.y;
    };
#pragma unroll 2
    for (int q = 0; q < 8; ++q) {
      const int src = 4 * q + grp;
      const uint32_t nt = __shfl_sync(0xffffffffu, nt_l, src);
      const uint32_t off = __shfl_sync(0xffffffffu, off_l, src);
      float v[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = 0.f;
      // slots r = sub, sub + 8, sub + 16, ... in order; unwritten slots are exact zeros
      if (marks & (1u << (2 * q))) add_record(v, off + sub);
      if (marks & (2u << (2 * q))) add_record(v, off + sub + 8);
      for (uint32_t r = sub + 16; r < nt; r += 8)
        if (a.written[off + r]) add_record(v, off + r);
      group8_sum16(v, lane);
      if (sub < 5) {
        s_acc[warp * 32 + src][2 * sub] = v[0];
        s_acc[warp * 32 + src][2 * sub + 1] = v[1];
      }
    }
  }
  __syncthreads();

  // ---- phase 2: one thread per Gaussian ----------------------------------------------
  bool sh_ready = true;
  if (bulk) {
    sh_ready = mbar_wait(bar, 0);
    if (!sh_ready) atomicOr(a.flags, CFGS_FLAG_COPY_TIMEOUT);
  }
  const int64_t idx = blk0 + threadIdx.x;
  const bool valid = idx < a.total_slots && idx - sd.gauss_base < sd.num_gaussians;
  const uint32_t nt = (valid && a.radii[idx] > 0) ? a.geom.touched[idx] : 0u;
  const bool want_dsh = !pose_only && a.out.dL_dsh != nullptr;
  float* own_sh = reinterpret_cast<float*>(s_sh + 12 * threadIdx.x);
  const float* sh_src = nullptr;
  float* dsh_dst = nullptr;
  if (idx < a.total_slots && a.g.shs) {
    sh_src = bulk && sh_ready ? own_sh : a.g.shs + (size_t)idx * 3 * M;
    if (want_dsh) dsh_dst = bulk ? own_sh : a.out.dL_dsh + (size_t)idx * 3 * M;
  }
  float dmean[3] = {0.f, 0.f, 0.f};
  if (idx < a.total_slots) {
    if (nt > 0) {
      float acc[10];
#pragma unroll
      for (int k = 0; k < 10; ++k) acc[k] = s_acc[threadIdx.x][k];
      gaussian_backward(a, sd, idx, nt, acc, sh_src, dsh_dst, pose_only, dmean);
    } else if (!pose_only) {
      zero_gradients(a, idx, M, dsh_dst);
    }
  }
  if (bulk && want_dsh) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(
                       a.out.dL_dsh + (size_t)blk0 * 3 * kMaxShCoeffs),
                   "r"(smem_addr(s_sh)), "r"(sh_bytes)
                   : "memory");
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
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
  {
    const double tot = warp_sum6_f64(term, lane);  // lane 4k: term k of the warp
    if ((lane & 3) == 0 && (lane >> 2) < 6) s_red[warp][lane >> 2] = tot;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double vv = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) vv += s_red[w][threadIdx.x];
    a.pose_partials[(size_t)blockIdx.x * 9 + threadIdx.x] = vv;
  } else if (threadIdx.x < 9) {
    a.pose_partials[(size_t)blockIdx.x * 9 + threadIdx.x] = 0.0;
  }
}

template <class Scenes>
void launch_preprocess_bwd(const PreBwdArgs<Scenes>& a, int blocks, cudaStream_t st) {
  constexpr int kShBulkBytes = 256 * 3 * kMaxShCoeffs * (int)sizeof(float);
  static std::atomic<uint64_t> smem_set{0}, smem_set_pose{0};
  // a failure of the attribute call surfaces as a launch error
  if (a.pose_partials) {  // pose-only form: fewer live values, a fourth resident block per SM
    ensure_dynamic_smem(k_preprocess_bwd<Scenes, true>, kShBulkBytes, smem_set_pose);
    k_preprocess_bwd<Scenes, true><<<blocks, 256, a.sh_bulk ? kShBulkBytes : 0, st>>>(a);
  } else {
    ensure_dynamic_smem(k_preprocess_bwd<Scenes, false>, kShBulkBytes, smem_set);
    k_preprocess_bwd<Scenes, false><<<blocks, 256, a.sh_bulk ? kShBulkBytes : 0, st>>>(a);
  }
}
template void launch_preprocess_bwd<SingleScene>(const PreBwdArgs<SingleScene>&, int, cudaStream_t);
template void launch_preprocess_bwd<SceneTable>(const PreBwdArgs<SceneTable>&, int, cudaStream_t);

}  // namespace cfgs

// ---- diagnostics: the bounded copy wait --------------------------------------------
namespace cfgs {

// One thread arms an mbarrier for `bytes` of transfer that no copy ever delivers and
// waits on it with the library's bounded wait (max_polls polls), exactly as the kernels
// wait for their bulk and tensor copies; when the wait gives up it raises
// CFGS_FLAG_COPY_TIMEOUT in *flags. No copy is issued, so nothing is in flight when the
// block exits.
__global__ void __launch_bounds__(32) k_copy_wait_diag(uint32_t max_polls, uint32_t bytes, uint32_t* flags) {
  __shared__ __align__(8) uint64_t s_bar;
  if (threadIdx.x != 0) return;
  const uint32_t bar = smem_addr(&s_bar);
  mbar_init(bar, 1);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  if (!mbar_wait(bar, 0, max_polls)) atomicOr(flags, CFGS_FLAG_COPY_TIMEOUT);
}

}  // namespace cfgs

extern "C" int cfgs_diag_copy_timeout(uint32_t max_polls, uint32_t* flags, void* stream) {
  if (!flags || max_polls == 0 || max_polls > cfgs::kMbarMaxPolls) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(flags, 0, sizeof(uint32_t), st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  cfgs::k_copy_wait_diag<<<1, 32, 0, st>>>(max_polls, 1024u, flags);
  if (cudaGetLastError() != cudaSuccess) return CFGS_ERR_LAUNCH;
  uint32_t host = 0;
  if (cudaMemcpyAsync(&host, flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CFGS_ERR_LAUNCH;
  return (host & CFGS_FLAG_COPY_TIMEOUT) ? CFGS_ERR_DEVICE_FLAG : CFGS_OK;
}
