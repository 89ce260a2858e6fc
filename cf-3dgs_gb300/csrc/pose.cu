// CF-3DGS relative-pose path: SE(3) retraction applied to the Gaussians, the fused
// pose-gradient reduction, and the Adam step on the 6-vector tangent.
//
// Parametrisation (the one lietorch's LieGroupParameter(SE3) gives CFGaussianModel,
// scene/gaussian_model_cf.py:123-133 and :328-340): the optimised tensor is a tangent
// xi = (rho, phi) in R^6, initialised at 0; the pose is X = exp(xi) * I with
// R = exp(phi^) and t = J_l(phi) rho (J_l = SO(3) left Jacobian); positions move as
// p' = R p + t. Covariances are not moved by the reference pose
// (scene/gaussian_model_cf.py:119-121); the rotate_cov form (cov' = R cov R^T) is an
// option of this library.
//
// Gradient. With a left perturbation exp(d) X of the pose, dL/dd = (sum g_i,
// sum p'_i x g_i + w_cov), where g_i = dL/dp'_i and w_cov is the rotation gradient of
// the rotated covariances. Since exp(xi + dxi) = exp(J(xi) dxi) exp(xi) with J the
// SE(3) left Jacobian, dL/dxi = J(xi)^T dL/dd. The kernel forms the sums in one pass
// over the Gaussians; the last block to finish adds the per-block partials in block
// order (deterministic) and applies J^T in double precision.
#include "cfgs_internal.cuh"

namespace cfgs {

constexpr int kPoseThreads = 256;
constexpr int kPoseMaxBlocks = 1184;  // 152 SMs x 8 blocks
constexpr int kPosePartials = 9;      // sum g (3), sum (R p) x g (3), w_cov (3)

struct SE3d {
  double R[9];
  double t[3];
};

__host__ __device__ inline void hat(const double* w, double* M) {
  M[0] = 0;     M[1] = -w[2]; M[2] = w[1];
  M[3] = w[2];  M[4] = 0;     M[5] = -w[0];
  M[6] = -w[1]; M[7] = w[0];  M[8] = 0;
}
__host__ __device__ inline void mm3(const double* A, const double* B, double* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}

// Coefficients of exp / left Jacobian as functions of theta, with series near 0.
__device__ inline void so3_coeffs(double th2, double* a, double* b, double* c) {
  // a = sin(th)/th, b = (1-cos th)/th^2, c = (th - sin th)/th^3
  if (th2 < 1e-8) {
    *a = 1.0 - th2 / 6.0;
    *b = 0.5 - th2 / 24.0;
    *c = 1.0 / 6.0 - th2 / 120.0;
  } else {
    double th = sqrt(th2);
    double s = sin(th), co = cos(th);
    *a = s / th;
    *b = (1.0 - co) / th2;
    *c = (th - s) / (th2 * th);
  }
}

__device__ inline void se3_exp(const float* xi, SE3d* X, double* Jl) {
  double rho[3] = {xi[0], xi[1], xi[2]};
  double phi[3] = {xi[3], xi[4], xi[5]};
  double th2 = phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2];
  double a, b, c;
  so3_coeffs(th2, &a, &b, &c);
  double P[9], P2[9];
  hat(phi, P);
  mm3(P, P, P2);
  for (int k = 0; k < 9; ++k) {
    double I = (k % 4 == 0) ? 1.0 : 0.0;
    X->R[k] = I + a * P[k] + b * P2[k];
    Jl[k] = I + b * P[k] + c * P2[k];
  }
  for (int i = 0; i < 3; ++i) X->t[i] = Jl[3 * i] * rho[0] + Jl[3 * i + 1] * rho[1] + Jl[3 * i + 2] * rho[2];
}

// Q(rho, phi): the upper-right block of the SE(3) left Jacobian (Barfoot, "State
// Estimation for Robotics", eq. 7.86).
__device__ inline void se3_Q(const double* rho, const double* phi, double* Q) {
  double th2 = phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2];
  double c1, c2, c3;
  if (th2 < 1e-6) {
    c1 = 1.0 / 6.0 - th2 / 120.0;
    c2 = 1.0 / 24.0 - th2 / 720.0;
    c3 = 1.0 / 120.0 - th2 / 2520.0;
  } else {
    double th = sqrt(th2), s = sin(th), co = cos(th);
    double th3 = th2 * th, th4 = th2 * th2, th5 = th4 * th;
    c1 = (th - s) / th3;
    c2 = (th2 + 2.0 * co - 2.0) / (2.0 * th4);
    c3 = (2.0 * th - 3.0 * s + th * co) / (2.0 * th5);
  }
  double Rh[9], Ph[9], PR[9], RP[9], PRP[9], PP[9], PPR[9], RPP[9], PRPP[9], PPRP[9];
  hat(rho, Rh);
  hat(phi, Ph);
  mm3(Ph, Rh, PR);
  mm3(Rh, Ph, RP);
  mm3(PR, Ph, PRP);
  mm3(Ph, Ph, PP);
  mm3(PP, Rh, PPR);
  mm3(Rh, PP, RPP);
  mm3(PRP, Ph, PRPP);
  mm3(Ph, PRP, PPRP);
  for (int k = 0; k < 9; ++k)
    Q[k] = 0.5 * Rh[k] + c1 * (PR[k] + RP[k] + PRP[k]) + c2 * (PPR[k] + RPP[k] - 3.0 * PRP[k]) +
           c3 * (PRPP[k] + PPRP[k]);
}

__global__ void __launch_bounds__(kPoseThreads) k_pose_apply(int n, const float* xi, const float* xyz,
                                                              const float* cov_in, float* means_out,
                                                              float* cov_out) {
  __shared__ float sR[9], st[3];
  if (threadIdx.x == 0) {
    SE3d X;
    double Jl[9];
    se3_exp(xi, &X, Jl);
    for (int k = 0; k < 9; ++k) sR[k] = (float)X.R[k];
    for (int k = 0; k < 3; ++k) st[k] = (float)X.t[k];
  }
  __syncthreads();
  float R[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = sR[k];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float p0 = xyz[3 * i], p1 = xyz[3 * i + 1], p2 = xyz[3 * i + 2];
#pragma unroll
    for (int r = 0; r < 3; ++r)  // ((R0 x + R1 y) + R2 z) + t, each operation rounded once
      means_out[3 * i + r] = __fadd_rn(
          __fadd_rn(__fadd_rn(__fmul_rn(R[3 * r], p0), __fmul_rn(R[3 * r + 1], p1)), __fmul_rn(R[3 * r + 2], p2)),
          st[r]);
    if (cov_in) {
      const float* c = cov_in + 6 * (size_t)i;
      float C[9] = {c[0], c[1], c[2], c[1], c[3], c[4], c[2], c[4], c[5]};
      float RC[9];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) RC[3 * a + b] = R[3 * a] * C[b] + R[3 * a + 1] * C[3 + b] + R[3 * a + 2] * C[6 + b];
      const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        int a = ii[k], b = jj[k];
        cov_out[6 * (size_t)i + k] = RC[3 * a] * R[3 * b] + RC[3 * a + 1] * R[3 * b + 1] + RC[3 * a + 2] * R[3 * b + 2];
      }
    }
  }
}

// dL/dxi from the left-perturbation sums tot = (sum g, sum (R p) x g, w_cov):
// d_rho = sum g, d_phi = sum (R p + t) x g + w_cov, then dL/dxi = J^T dL/dd with the
// SE(3) left Jacobian J = [[Jl, Q], [0, Jl]] — all in float64, rounded at the end.
__device__ void pose_grad_from_sums(const float* xi, const double* tot, float* grad_out) {
  SE3d X;
  double Jl[9], Q[9];
  se3_exp(xi, &X, Jl);
  double rho[3] = {xi[0], xi[1], xi[2]};
  double phi[3] = {xi[3], xi[4], xi[5]};
  se3_Q(rho, phi, Q);
  double gr[3] = {tot[0], tot[1], tot[2]};
  double gp[3];
  gp[0] = tot[3] + (X.t[1] * gr[2] - X.t[2] * gr[1]) + tot[6];
  gp[1] = tot[4] + (X.t[2] * gr[0] - X.t[0] * gr[2]) + tot[7];
  gp[2] = tot[5] + (X.t[0] * gr[1] - X.t[1] * gr[0]) + tot[8];
  for (int j = 0; j < 3; ++j) {
    grad_out[j] = (float)(Jl[j] * gr[0] + Jl[3 + j] * gr[1] + Jl[6 + j] * gr[2]);
    grad_out[3 + j] = (float)(Q[j] * gr[0] + Q[3 + j] * gr[1] + Q[6 + j] * gr[2] + Jl[j] * gp[0] +
                              Jl[3 + j] * gp[1] + Jl[6 + j] * gp[2]);
  }
}

struct PoseGradArgs {
  int n;
  const float* xi;
  const float* xyz;
  const float* dL_dmeans;
  const float* cov_rot;
  const float* dL_dcov;
  double* partials;       // [gridDim.x][9]
  unsigned int* counter;  // zeroed before launch
  float* grad_out;        // [6]
};

// Sums in float64: the per-Gaussian terms (R p) x g use the float64 rotation and
// exact float32 x float32 products, so the result is the float64 value of the same
// sums a float64 autograd of exp(xi).act(p) forms; rounded to float32 at the end, the
// gradient then matches that path's in all but boundary cases, which keeps the fused
// and plain solves on the same trajectory.
__global__ void __launch_bounds__(kPoseThreads) k_pose_grad(PoseGradArgs a) {
  __shared__ double sR[9];
  __shared__ double s_red[kPoseThreads / 32][kPosePartials];
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    SE3d X;
    double Jl[9];
    se3_exp(a.xi, &X, Jl);
    for (int k = 0; k < 9; ++k) sR[k] = X.R[k];
  }
  __syncthreads();
  double R[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = sR[k];
  double acc[kPosePartials];
#pragma unroll
  for (int k = 0; k < kPosePartials; ++k) acc[k] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    double p0 = a.xyz[3 * i], p1 = a.xyz[3 * i + 1], p2 = a.xyz[3 * i + 2];
    double g0 = a.dL_dmeans[3 * i], g1 = a.dL_dmeans[3 * i + 1], g2 = a.dL_dmeans[3 * i + 2];
    double q0 = R[0] * p0 + R[1] * p1 + R[2] * p2;
    double q1 = R[3] * p0 + R[4] * p1 + R[5] * p2;
    double q2 = R[6] * p0 + R[7] * p1 + R[8] * p2;
    acc[0] += g0;
    acc[1] += g1;
    acc[2] += g2;
    acc[3] += q1 * g2 - q2 * g1;
    acc[4] += q2 * g0 - q0 * g2;
    acc[5] += q0 * g1 - q1 * g0;
    if (a.cov_rot) {
      const float* c = a.cov_rot + 6 * (size_t)i;
      const float* d = a.dL_dcov + 6 * (size_t)i;
      float C[9] = {c[0], c[1], c[2], c[1], c[3], c[4], c[2], c[4], c[5]};
      float G[9] = {d[0], 0.5f * d[1], 0.5f * d[2], 0.5f * d[1], d[3], 0.5f * d[4], 0.5f * d[2], 0.5f * d[4], d[5]};
      // M = C G - G C (antisymmetric); w = (M12 - M21, M20 - M02, M01 - M10) = 2 (M12, M20, M01)
      float CG[9];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int s = 0; s < 3; ++s) CG[3 * r + s] = C[3 * r] * G[s] + C[3 * r + 1] * G[3 + s] + C[3 * r + 2] * G[6 + s];
      // (G C) = (C G)^T for symmetric C, G, so M_rs = CG_rs - CG_sr.
      acc[6] += 2.0 * ((double)CG[5] - (double)CG[7]);
      acc[7] += 2.0 * ((double)CG[6] - (double)CG[2]);
      acc[8] += 2.0 * ((double)CG[1] - (double)CG[3]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kPosePartials; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < kPosePartials) {
    double v = 0.0;
    for (int w = 0; w < kPoseThreads / 32; ++w) v += s_red[w][threadIdx.x];
    a.partials[blockIdx.x * kPosePartials + threadIdx.x] = v;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    double tot[kPosePartials];
    for (int k = 0; k < kPosePartials; ++k) tot[k] = 0.0;
    const volatile double* part = a.partials;
    for (int b = 0; b < (int)gridDim.x; ++b)
      for (int k = 0; k < kPosePartials; ++k) tot[k] += part[b * kPosePartials + k];
    pose_grad_from_sums(a.xi, tot, a.grad_out);
    *a.counter = 0u;
  }
}

// One Adam step on `count` 6-vectors (one per solve), following the operation sequence
// of torch.optim.Adam's default multi-tensor path for float32 CUDA tensors:
//   m = lerp(m, g, 1 - b1);  v = v * b2;  v = addcmul(v, g, g, 1 - b2);
//   denom = sqrt(v) / sqrt(1 - b2^t) + eps;  p = addcdiv(p, m, denom, -lr / (1 - b1^t))
// with the hyper-parameters as float64 scalars rounded to float32 per use, as torch
// passes them, so both optimisers take the same steps. bc1 = 1 - b1^t and
// bc2 = 1 - b2^t are float64, as torch forms them on the host.
// state per solve: m[6], v[6], step, 3 unused floats.
__device__ __forceinline__ double bias_correction(double beta, const float* st) {
  return 1.0 - pow(beta, (double)(st[12] + 1.0f));
}

__device__ void adam_step6_bc(float* xi, const float* grad, float* st, double lr, double b1, double b2, double eps,
                              double bc1, double bc2) {
  const float step = st[12] + 1.0f;
  const float w1 = (float)(1.0 - b1), mul2 = (float)b2, w2 = (float)(1.0 - b2);
  const float step_size = (float)(-(lr / bc1));
  const float bc2_sqrt = (float)sqrt(bc2);
  const float eps_f = (float)eps;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const float g = grad[k];
    float m = st[k], v = st[6 + k];
    m = fmaf(w1, g - m, m);
    v = v * mul2;
    v = fmaf(w2, g * g, v);
    st[k] = m;
    st[6 + k] = v;
    float denom = sqrtf(v) / bc2_sqrt;
    denom = denom + eps_f;
    xi[k] = fmaf(step_size, m / denom, xi[k]);
  }
  st[12] = step;
}

__device__ void adam_step6(float* xi, const float* grad, float* st, double lr, double b1, double b2, double eps) {
  adam_step6_bc(xi, grad, st, lr, b1, b2, eps, bias_correction(b1, st), bias_correction(b2, st));
}

__global__ void k_pose_adam(int count, float* xi, const float* grad, float* state, double lr, double b1, double b2,
                            double eps) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= count) return;
  adam_step6(xi + 6 * (size_t)s, grad + 6 * (size_t)s, state + 16 * (size_t)s, lr, b1, b2, eps);
}

// The parts of a solve's pose state that depend on xi, split so that two threads can
// form them at once: exp(xi) with the left Jacobian, and the Q block.
__device__ void pose_state_exp(const float* xi, PoseState* ps) {
  SE3d X;
  double Jl[9];
  se3_exp(xi, &X, Jl);
  for (int k = 0; k < 9; ++k) {
    ps->R64[k] = X.R[k];
    ps->R[k] = (float)X.R[k];
    ps->Jl[k] = Jl[k];
  }
  for (int k = 0; k < 3; ++k) {
    ps->t64[k] = X.t[k];
    ps->t[k] = (float)X.t[k];
  }
}

__device__ void pose_state_Q(const float* xi, PoseState* ps) {
  const double rho[3] = {xi[0], xi[1], xi[2]};
  const double phi[3] = {xi[3], xi[4], xi[5]};
  se3_Q(rho, phi, ps->Q);
}

// pose_grad_from_sums with exp(xi), Jl and Q taken from the solve's state.
__device__ void pose_grad_from_state(const PoseState& ps, const double* tot, float* grad_out) {
  const double gr[3] = {tot[0], tot[1], tot[2]};
  double gp[3];
  gp[0] = tot[3] + (ps.t64[1] * gr[2] - ps.t64[2] * gr[1]) + tot[6];
  gp[1] = tot[4] + (ps.t64[2] * gr[0] - ps.t64[0] * gr[2]) + tot[7];
  gp[2] = tot[5] + (ps.t64[0] * gr[1] - ps.t64[1] * gr[0]) + tot[8];
  const double* Jl = ps.Jl;
  const double* Q = ps.Q;
  for (int j = 0; j < 3; ++j) {
    grad_out[j] = (float)(Jl[j] * gr[0] + Jl[3 + j] * gr[1] + Jl[6 + j] * gr[2]);
    grad_out[3 + j] = (float)(Q[j] * gr[0] + Q[3 + j] * gr[1] + Q[6 + j] * gr[2] + Jl[j] * gp[0] +
                              Jl[3 + j] * gp[1] + Jl[6 + j] * gp[2]);
  }
}

// One block per solve: the state of xi (exp, Q, the next step's bias corrections) by
// four threads at once.
__global__ void k_batch_pose_init(const float* xi, const float* adam_state, PoseState* states, double b1,
                                  double b2) {
  const int s = blockIdx.x;
  const float* x = xi + 6 * (size_t)s;
  const float* st = adam_state + 16 * (size_t)s;
  switch (threadIdx.x) {
    case 0: pose_state_exp(x, states + s); break;
    case 32: pose_state_Q(x, states + s); break;
    case 64: states[s].bc1 = bias_correction(b1, st); break;
    case 96: states[s].bc2 = bias_correction(b2, st); break;
    default: break;
  }
}

// One block per solve: the solve's per-block pose partials summed in a fixed pattern
// (thread i takes blocks i, i+256, ...; then a fixed tree), the SE(3) Jacobian
// transpose and the Adam step with the state's cached Jacobian blocks and bias
// corrections, then the state of the new xi by four threads at once. A solve's result
// depends only on its own blocks, so it is the same whatever else is in the batch.
__global__ void __launch_bounds__(256) k_batch_pose_update(const SceneDesc* descs, const double* partials,
                                                           float* xi, float* adam_state, PoseState* states,
                                                           const CfgsCounts* counts, int64_t cap, double lr,
                                                           double b1, double b2, double eps) {
  __shared__ double s_red[8][6];
  __shared__ float s_x[6];
  if ((int64_t)counts->num_rendered > cap) return;  // overflowed iteration: no update
  const int s = blockIdx.x;
  const SceneDesc& sd = descs[s];
  const int b0 = sd.gauss_base / kPreprocessBlock;
  const int nb = (sd.num_gaussians + kPreprocessBlock - 1) / kPreprocessBlock;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < 6; ++k) acc[k] += partials[(size_t)(b0 + b) * 9 + k];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  {
    const double tot = warp_sum6_f64(acc, lane);  // lane 4k: partial k of the warp
    if ((lane & 3) == 0 && (lane >> 2) < 6) s_red[warp][lane >> 2] = tot;
  }
  __syncthreads();
  float* x = xi + 6 * (size_t)s;
  float* st = adam_state + 16 * (size_t)s;
  PoseState* ps = states + s;
  if (threadIdx.x == 0) {
    double tot[kPosePartials];
    for (int k = 0; k < kPosePartials; ++k) tot[k] = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      for (int k = 0; k < 6; ++k) tot[k] += s_red[w][k];
    float grad[6];
    pose_grad_from_state(*ps, tot, grad);
    adam_step6_bc(x, grad, st, lr, b1, b2, eps, ps->bc1, ps->bc2);
    for (int k = 0; k < 6; ++k) s_x[k] = x[k];
  }
  __syncthreads();
  switch (threadIdx.x) {
    case 0: pose_state_exp(s_x, ps); break;
    case 32: pose_state_Q(s_x, ps); break;
    case 64: ps->bc1 = bias_correction(b1, st); break;
    case 96: ps->bc2 = bias_correction(b2, st); break;
    default: break;
  }
}

void launch_batch_pose_init(int count, const float* xi, const float* adam_state, PoseState* states, double b1,
                            double b2, cudaStream_t st) {
  k_batch_pose_init<<<count, 128, 0, st>>>(xi, adam_state, states, b1, b2);
}
void launch_batch_pose_update(int count, const SceneDesc* descs, const double* partials, float* xi,
                              float* adam_state, PoseState* states, const CfgsCounts* counts, int64_t cap, double lr,
                              double b1, double b2, double eps, cudaStream_t st) {
  k_batch_pose_update<<<count, 256, 0, st>>>(descs, partials, xi, adam_state, states, counts, cap, lr, b1, b2, eps);
}

}  // namespace cfgs

using namespace cfgs;

static int pose_blocks(int n) {
  int b = div_up(n > 0 ? n : 1, kPoseThreads);
  return b < kPoseMaxBlocks ? b : kPoseMaxBlocks;
}

extern "C" int cfgs_pose_apply(int32_t n, const float* xi, const float* xyz, const float* cov_in, float* means_out,
                               float* cov_out, void* stream) {
  if (n < 0 || !xi || (n > 0 && (!xyz || !means_out))) return CFGS_ERR_INVALID_ARGUMENT;
  if ((cov_in == nullptr) != (cov_out == nullptr)) return CFGS_ERR_INVALID_ARGUMENT;
  if (n == 0) return CFGS_OK;
  k_pose_apply<<<pose_blocks(n), kPoseThreads, 0, (cudaStream_t)stream>>>(n, xi, xyz, cov_in, means_out, cov_out);
  CFGS_CHECK_LAUNCH(0, stream);
  return CFGS_OK;
}

extern "C" size_t cfgs_pose_scratch_bytes(int32_t n) {
  (void)n;
  return align256(sizeof(double) * kPosePartials * kPoseMaxBlocks) + 256;
}

extern "C" int cfgs_pose_grad(int32_t n, const float* xi, const float* xyz, const float* dL_dmeans, const float* cov_rot,
                              const float* dL_dcov, void* scratch, float* grad_out, void* stream) {
  if (n < 0 || !xi || !scratch || !grad_out || (n > 0 && (!xyz || !dL_dmeans))) return CFGS_ERR_INVALID_ARGUMENT;
  if ((cov_rot == nullptr) != (dL_dcov == nullptr)) return CFGS_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  PoseGradArgs a;
  a.n = n;
  a.xi = xi;
  a.xyz = xyz;
  a.dL_dmeans = dL_dmeans;
  a.cov_rot = cov_rot;
  a.dL_dcov = dL_dcov;
  a.partials = static_cast<double*>(scratch);
  a.counter = reinterpret_cast<unsigned int*>(static_cast<char*>(scratch) +
                                              align256(sizeof(double) * kPosePartials * kPoseMaxBlocks));
  a.grad_out = grad_out;
  if (cudaMemsetAsync(a.counter, 0, sizeof(unsigned int), st) != cudaSuccess) return CFGS_ERR_LAUNCH;
  k_pose_grad<<<pose_blocks(n), kPoseThreads, 0, st>>>(a);
  CFGS_CHECK_LAUNCH(0, st);
  return CFGS_OK;
}

extern "C" int cfgs_pose_adam(int32_t count, float* xi, const float* grad, float* state, double lr, double beta1,
                              double beta2, double eps, void* stream) {
  if (count < 0 || (count > 0 && (!xi || !grad || !state))) return CFGS_ERR_INVALID_ARGUMENT;
  if (count == 0) return CFGS_OK;
  k_pose_adam<<<div_up(count, 128), 128, 0, (cudaStream_t)stream>>>(count, xi, grad, state, lr, beta1, beta2, eps);
  CFGS_CHECK_LAUNCH(0, stream);
  return CFGS_OK;
}
