/*
 * CPU oracle of the differentiable Gaussian rasteriser — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * library, and only as the checker; the product path never calls it.
 *
 * It restates the published 3DGS rasteriser that CF-3DGS calls through
 * `diff_gaussian_rasterization` (un-vendored submodule, .gitmodules:4-6; call sites
 * scene/gaussian_model_cf.py:811-884, gaussian_renderer/__init__.py:38-96) in the
 * upstream algorithm's own shape:
 *   preprocess per Gaussian  -> inclusive scan of tiles touched
 *   -> duplicateWithKeys: key = tile << 32 | depth bits, value = Gaussian id, in
 *      Gaussian order and row-major over the tile rectangle
 *   -> stable LSD radix sort of the 64-bit keys -> identifyTileRanges
 *   -> per-pixel front-to-back compositing -> backward by back-to-front replay.
 * The in-tree Python math it follows: utils/general_utils.py:76-108 (covariance from
 * scale and quaternion), utils/sh_utils.py:26-112 (SH basis and constants),
 * scene/cameras.py:57-74 + utils/graphics_utils.py:57-113 (camera matrices).
 *
 * Float rounding. The forward uses float32 with exactly the operation sequence the GPU
 * kernels use (each a*b, a+b, a/b, sqrtf rounded once; fmaf where the kernel fuses), so
 * radii, tile rectangles, depth keys, tile ranges, contributor counts and the image
 * agree bit for bit. It must be compiled without FMA contraction (-ffp-contract=off).
 * exp() is the project's own Cody-Waite + degree-7 Taylor evaluation, identical to the
 * kernel's. The backward accumulates in double.
 *
 * Parity pinning: the SH, covariance and camera pieces are checked against fixtures
 * generated by running the reference's own Python functions (tests/golden/). The
 * compositing and sort semantics follow the published algorithm; the reference CUDA
 * source is not in the reference tree, so that part is unpinned against it.
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TILE 16
#define ALPHA_MAX 0.99f
#define ALPHA_MIN 0.003921568859368563f
#define T_MIN 0.0001f
#define NEAR_Z 0.2f

static const float SH_C0 = 0.28209479177387814f;
static const float SH_C1 = 0.4886025119029199f;
static const float SH_C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                               -1.0925484305920792f, 0.5462742152960396f};
static const float SH_C3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                               0.3731763325901154f, -0.4570457994644658f, 1.445305721320277f,
                               -0.5900435899266435f};

typedef struct {
  int H, W;
  float tanfovx, tanfovy;
  const float* bg;     /* [3] */
  float scale_modifier;
  const float* view;   /* [16] */
  const float* proj;   /* [16] */
  int sh_degree;
  const float* campos; /* [3] */
} OSettings;

typedef struct {
  int N;
  const float* means3D;
  const float* opac;
  const float* shs;
  int M;
  const float* colors;
  const float* scales;
  const float* rots;
  const float* cov3D;
} OGauss;

/* Per-Gaussian results of the preprocess. */
typedef struct {
  int32_t* radii;     /* [N] */
  float* xy;          /* [N,2] */
  float* conic_op;    /* [N,4] */
  float* rgbd;        /* [N,4] */
  int32_t* rect;      /* [N,4] min_x, min_y, max_x, max_y */
  uint32_t* touched;  /* [N] */
  uint8_t* clamped;   /* [N] */
} OGeom;

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* ---- scalar helpers -------------------------------------------------------------- */

static float f_from_bits(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static uint32_t bits_of(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

/* float -> int32 truncating toward zero, saturating, NaN -> 0 (the GPU's cvt.rzi). */
static int f2i(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT_MAX;
  if (f <= -2147483648.0f) return INT_MIN;
  return (int)f;
}

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* The project's exp: x = k ln2 + r, ln2 = head (15 significant bits) + tail, e^r by
 * the degree-7 Taylor polynomial in Horner form, exact scaling by 2^k in two steps. */
float oracle_exp(float x) {
  if (x != x) return x;
  if (x < -104.0f) return 0.0f;
  if (x > 88.75f) return f_from_bits(0x7f800000u);
  const float log2e = 1.4426950216293335f;
  const float ln2_hi = 0.693145751953125f;
  const float ln2_lo = 1.428606765330187e-06f;
  float kf = rintf(x * log2e);
  float r = fmaf(-kf, ln2_hi, x);
  r = fmaf(-kf, ln2_lo, r);
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
  float s1 = f_from_bits((uint32_t)(k1 + 127) << 23);
  float s2 = f_from_bits((uint32_t)(k2 + 127) << 23);
  return (p * s1) * s2;
}

/* [p,1] @ M (row-vector convention), accumulated m[12] -> +x -> +y -> +z. */
static void xform43(const float* m, const float* p, float* r) {
  r[0] = fmaf(m[8], p[2], fmaf(m[4], p[1], fmaf(m[0], p[0], m[12])));
  r[1] = fmaf(m[9], p[2], fmaf(m[5], p[1], fmaf(m[1], p[0], m[13])));
  r[2] = fmaf(m[10], p[2], fmaf(m[6], p[1], fmaf(m[2], p[0], m[14])));
}
static float xform_w(const float* m, const float* p) {
  return fmaf(m[11], p[2], fmaf(m[7], p[1], fmaf(m[3], p[0], m[15])));
}

/* Sigma = R S S R^T, R from quaternion (r,x,y,z) as utils/general_utils.py:76-97 builds
 * it, S = diag(mod * s) as build_scaling_rotation (:99-108); stored as
 * strip_symmetric (:62-74) does: (xx, xy, xz, yy, yz, zz). */
static void cov3d(const float* s, float mod, const float* q, float* cov) {
  float sx = mod * s[0], sy = mod * s[1], sz = mod * s[2];
  float r = q[0], x = q[1], y = q[2], z = q[3];
  float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
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
  for (int i = 0; i < 3; ++i) {
    M[3 * i + 0] = R[3 * i + 0] * sx;
    M[3 * i + 1] = R[3 * i + 1] * sy;
    M[3 * i + 2] = R[3 * i + 2] * sz;
  }
  static const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
  for (int k = 0; k < 6; ++k) {
    const float* a = M + 3 * ii[k];
    const float* b = M + 3 * jj[k];
    cov[k] = fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0]));
  }
}

/* EWA: cov2D = J W Sigma W^T J^T + 0.3 I, J clamped at 1.3 tan(fov). */
static void cov2d(const float* t, float fx, float fy, float tanfovx, float tanfovy, const float* cov,
                  const float* V, float* out) {
  float limx = 1.3f * tanfovx, limy = 1.3f * tanfovy;
  float txtz = t[0] / t[2], tytz = t[1] / t[2];
  float tx = fminf(limx, fmaxf(-limx, txtz)) * t[2];
  float ty = fminf(limy, fmaxf(-limy, tytz)) * t[2];
  float tz2 = t[2] * t[2];
  float J00 = fx / t[2];
  float J02 = -(fx * tx) / tz2;
  float J11 = fy / t[2];
  float J12 = -(fy * ty) / tz2;
  float T0[3], T1[3];
  for (int j = 0; j < 3; ++j) {
    T0[j] = fmaf(J02, V[4 * j + 2], J00 * V[4 * j + 0]);
    T1[j] = fmaf(J12, V[4 * j + 2], J11 * V[4 * j + 1]);
  }
  float S[9] = {cov[0], cov[1], cov[2], cov[1], cov[3], cov[4], cov[2], cov[4], cov[5]};
  float u[3], v[3];
  for (int i = 0; i < 3; ++i) {
    u[i] = fmaf(S[3 * i + 2], T0[2], fmaf(S[3 * i + 1], T0[1], S[3 * i + 0] * T0[0]));
    v[i] = fmaf(S[3 * i + 2], T1[2], fmaf(S[3 * i + 1], T1[1], S[3 * i + 0] * T1[0]));
  }
  float a = fmaf(T0[2], u[2], fmaf(T0[1], u[1], T0[0] * u[0]));
  float b = fmaf(T0[2], v[2], fmaf(T0[1], v[1], T0[0] * v[0]));
  float c = fmaf(T1[2], v[2], fmaf(T1[1], v[1], T1[0] * v[0]));
  out[0] = a + 0.3f;
  out[1] = b;
  out[2] = c + 0.3f;
}

static float ndc2pix(float v, int S) { return ((v + 1.0f) * (float)S - 1.0f) * 0.5f; }

/* SH basis values at unit direction (x,y,z) for degree <= 3 (utils/sh_utils.py:57-105). */
static int sh_basis(int deg, float x, float y, float z, float* b) {
  b[0] = SH_C0;
  if (deg < 1) return 1;
  b[1] = -SH_C1 * y;
  b[2] = SH_C1 * z;
  b[3] = -SH_C1 * x;
  if (deg < 2) return 4;
  float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  b[4] = SH_C2[0] * xy;
  b[5] = SH_C2[1] * yz;
  b[6] = SH_C2[2] * ((2.0f * zz - xx) - yy);
  b[7] = SH_C2[3] * xz;
  b[8] = SH_C2[4] * (xx - yy);
  if (deg < 3) return 9;
  b[9] = (SH_C3[0] * y) * (3.0f * xx - yy);
  b[10] = (SH_C3[1] * xy) * z;
  b[11] = (SH_C3[2] * y) * ((4.0f * zz - xx) - yy);
  b[12] = (SH_C3[3] * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
  b[13] = (SH_C3[4] * x) * ((4.0f * zz - xx) - yy);
  b[14] = (SH_C3[5] * z) * (xx - yy);
  b[15] = (SH_C3[6] * x) * (xx - 3.0f * yy);
  return 16;
}

static void sh_rgb(int deg, const float* sh, const float* p, const float* campos, float* rgb, uint8_t* clamped) {
  float dx = p[0] - campos[0], dy = p[1] - campos[1], dz = p[2] - campos[2];
  float len = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
  float x = dx / len, y = dy / len, z = dz / len;
  float b[16];
  int nb = sh_basis(deg, x, y, z, b);
  float c[3];
  for (int ch = 0; ch < 3; ++ch) c[ch] = b[0] * sh[ch];
  for (int k = 1; k < nb; ++k)
    for (int ch = 0; ch < 3; ++ch) c[ch] = fmaf(b[k], sh[3 * k + ch], c[ch]);
  uint8_t cl = 0;
  for (int ch = 0; ch < 3; ++ch) {
    c[ch] = c[ch] + 0.5f;
    if (c[ch] < 0.0f) cl |= (uint8_t)(1u << ch);
    rgb[ch] = fmaxf(c[ch], 0.0f);
  }
  *clamped = cl;
}

/* ---- forward ----------------------------------------------------------------------- */

/* Preprocess every Gaussian. Returns K = total tiles touched (capped at 2^31 - 1). */
int64_t oracle_preprocess(const OSettings* s, const OGauss* g, OGeom* o) {
  const int gx = (s->W + TILE - 1) / TILE, gy = (s->H + TILE - 1) / TILE;
  const float fx = (float)s->W / (2.0f * s->tanfovx);
  const float fy = (float)s->H / (2.0f * s->tanfovy);
  int64_t K = 0;
#pragma omp parallel for schedule(static) reduction(+ : K)
  for (int i = 0; i < g->N; ++i) {
    o->radii[i] = 0;
    o->touched[i] = 0;
    o->clamped[i] = 0;
    for (int k = 0; k < 4; ++k) o->rect[4 * i + k] = 0;
    const float* p = g->means3D + 3 * (size_t)i;
    float t[3];
    xform43(s->view, p, t);
    if (t[2] <= NEAR_Z) continue;
    float hom[3];
    xform43(s->proj, p, hom);
    float hw = xform_w(s->proj, p);
    float w_inv = 1.0f / (hw + 0.0000001f);
    float proj[2] = {hom[0] * w_inv, hom[1] * w_inv};
    float cov[6];
    if (g->cov3D) {
      for (int k = 0; k < 6; ++k) cov[k] = g->cov3D[6 * (size_t)i + k];
    } else {
      cov3d(g->scales + 3 * (size_t)i, s->scale_modifier, g->rots + 4 * (size_t)i, cov);
    }
    float c2[3];
    cov2d(t, fx, fy, s->tanfovx, s->tanfovy, cov, s->view, c2);
    float det = c2[0] * c2[2] - c2[1] * c2[1];
    if (det == 0.0f) continue;
    float det_inv = 1.0f / det;
    float conic[3] = {c2[2] * det_inv, -c2[1] * det_inv, c2[0] * det_inv};
    float mid = 0.5f * (c2[0] + c2[2]);
    float disc = sqrtf(fmaxf(0.1f, mid * mid - det));
    float l1 = mid + disc, l2 = mid - disc;
    int rad = f2i(ceilf(3.0f * sqrtf(fmaxf(l1, l2))));
    float px = ndc2pix(proj[0], s->W), py = ndc2pix(proj[1], s->H);
    float rf = (float)rad;
    int x0 = imin(gx, imax(0, f2i((px - rf) / (float)TILE)));
    int y0 = imin(gy, imax(0, f2i((py - rf) / (float)TILE)));
    int x1 = imin(gx, imax(0, f2i(((px + rf) + (float)(TILE - 1)) / (float)TILE)));
    int y1 = imin(gy, imax(0, f2i(((py + rf) + (float)(TILE - 1)) / (float)TILE)));
    int area = (x1 - x0) * (y1 - y0);
    if (area == 0) continue;
    float rgb[3];
    uint8_t cl = 0;
    if (g->colors) {
      for (int ch = 0; ch < 3; ++ch) rgb[ch] = g->colors[3 * (size_t)i + ch];
    } else {
      sh_rgb(s->sh_degree, g->shs + (size_t)i * g->M * 3, p, s->campos, rgb, &cl);
    }
    o->radii[i] = rad;
    o->xy[2 * i] = px;
    o->xy[2 * i + 1] = py;
    o->conic_op[4 * i + 0] = conic[0];
    o->conic_op[4 * i + 1] = conic[1];
    o->conic_op[4 * i + 2] = conic[2];
    o->conic_op[4 * i + 3] = g->opac[i];
    o->rgbd[4 * i + 0] = rgb[0];
    o->rgbd[4 * i + 1] = rgb[1];
    o->rgbd[4 * i + 2] = rgb[2];
    o->rgbd[4 * i + 3] = t[2];
    o->rect[4 * i + 0] = x0;
    o->rect[4 * i + 1] = y0;
    o->rect[4 * i + 2] = x1;
    o->rect[4 * i + 3] = y1;
    o->touched[i] = (uint32_t)area;
    o->clamped[i] = cl;
    K += area;
  }
  return K;
}

/* Stable LSD radix sort of (key, value) pairs on the low `bits` bits of key. */
static void radix_sort_pairs(uint64_t* key, uint32_t* val, int64_t n, int bits) {
  uint64_t* k2 = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(n > 0 ? n : 1));
  uint32_t* v2 = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
  uint64_t *ks = key, *kd = k2;
  uint32_t *vs = val, *vd = v2;
  for (int shift = 0; shift < bits; shift += 8) {
    int64_t cnt[257];
    memset(cnt, 0, sizeof(cnt));
    for (int64_t i = 0; i < n; ++i) cnt[((ks[i] >> shift) & 255u) + 1]++;
    for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
    for (int64_t i = 0; i < n; ++i) {
      int64_t pos = cnt[(ks[i] >> shift) & 255u]++;
      kd[pos] = ks[i];
      vd[pos] = vs[i];
    }
    uint64_t* tk = ks; ks = kd; kd = tk;
    uint32_t* tv = vs; vs = vd; vd = tv;
  }
  if (ks != key) {
    memcpy(key, ks, sizeof(uint64_t) * (size_t)n);
    memcpy(val, vs, sizeof(uint32_t) * (size_t)n);
  }
  free(k2);
  free(v2);
}

/* duplicateWithKeys + stable sort + identifyTileRanges.
 * keys_out/gid_out: [K] sorted; ranges: [num_tiles + 1]. */
void oracle_bin(const OSettings* s, int N, const OGeom* o, int64_t K, uint64_t* keys_out, uint32_t* gid_out,
                uint32_t* ranges) {
  const int gx = (s->W + TILE - 1) / TILE, gy = (s->H + TILE - 1) / TILE;
  const int T = gx * gy;
  int64_t* off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N + 1));
  off[0] = 0;
  for (int i = 0; i < N; ++i) off[i + 1] = off[i] + o->touched[i];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; ++i) {
    if (!o->touched[i]) continue;
    int64_t j = off[i];
    uint64_t d = bits_of(o->rgbd[4 * i + 3]);
    for (int y = o->rect[4 * i + 1]; y < o->rect[4 * i + 3]; ++y)
      for (int x = o->rect[4 * i + 0]; x < o->rect[4 * i + 2]; ++x, ++j) {
        keys_out[j] = ((uint64_t)(uint32_t)(y * gx + x) << 32) | d;
        gid_out[j] = (uint32_t)i;
      }
  }
  free(off);
  int tile_bits = 0;
  while ((1 << tile_bits) < T + 1) ++tile_bits;
  radix_sort_pairs(keys_out, gid_out, K, 32 + tile_bits);
  for (int t = 0; t <= T; ++t) ranges[t] = 0;
  /* ranges[t] = first sorted position of tile t; ranges[T] = K (tiles without
   * instances get an empty range at the position of the next tile). */
  int64_t p = 0;
  for (int t = 0; t < T; ++t) {
    ranges[t] = (uint32_t)p;
    while (p < K && (int)(keys_out[p] >> 32) == t) ++p;
  }
  ranges[T] = (uint32_t)K;
}

/* Front-to-back compositing, one pixel at a time. */
void oracle_render(const OSettings* s, const OGeom* o, const uint32_t* gid, const uint32_t* ranges, float* out_color,
                   float* out_depth, float* out_alpha, float* final_T, uint32_t* n_contrib) {
  const int gx = (s->W + TILE - 1) / TILE, gy = (s->H + TILE - 1) / TILE;
  const size_t HW = (size_t)s->W * s->H;
#pragma omp parallel for schedule(dynamic, 4)
  for (int tile = 0; tile < gx * gy; ++tile) {
    const int tx = tile % gx, ty = tile / gx;
    for (int ly = 0; ly < TILE; ++ly)
      for (int lx = 0; lx < TILE; ++lx) {
        int px = tx * TILE + lx, py = ty * TILE + ly;
        if (px >= s->W || py >= s->H) continue;
        float pxf = (float)px, pyf = (float)py;
        float T = 1.0f, C[3] = {0, 0, 0}, D = 0.0f;
        uint32_t contributor = 0, last = 0;
        for (uint32_t i = ranges[tile]; i < ranges[tile + 1]; ++i) {
          ++contributor;
          uint32_t g = gid[i];
          float ca = -0.5f * o->conic_op[4 * g + 0];
          float cb = -o->conic_op[4 * g + 1];
          float cc = -0.5f * o->conic_op[4 * g + 2];
          float op = o->conic_op[4 * g + 3];
          float dx = o->xy[2 * g] - pxf, dy = o->xy[2 * g + 1] - pyf;
          float e = cb * (dx * dy);
          e = fmaf(cc * dy, dy, e);
          float power = fmaf(ca * dx, dx, e);
          if (power > 0.0f) continue;
          float alpha = fminf(ALPHA_MAX, op * oracle_exp(power));
          if (alpha < ALPHA_MIN) continue;
          float test_T = T * (1.0f - alpha);
          if (test_T < T_MIN) break;
          float w = alpha * T;
          for (int ch = 0; ch < 3; ++ch) C[ch] = fmaf(o->rgbd[4 * g + ch], w, C[ch]);
          D = fmaf(o->rgbd[4 * g + 3], w, D);
          T = test_T;
          last = contributor;
        }
        size_t pix = (size_t)py * s->W + px;
        final_T[pix] = T;
        n_contrib[pix] = last;
        for (int ch = 0; ch < 3; ++ch) out_color[ch * HW + pix] = fmaf(T, s->bg[ch], C[ch]);
        out_depth[pix] = D;
        out_alpha[pix] = 1.0f - T;
      }
  }
}

/* ---- backward ---------------------------------------------------------------------- */

/* Per-Gaussian gradients of the render: dxy (pixel space, 2), dconic (3), dopacity,
 * drgb (3), ddepth — accumulated in double into g10 [N,10]. */
void oracle_render_backward(const OSettings* s, int N, const OGeom* o, const uint32_t* gid, const uint32_t* ranges,
                            const float* final_T, const uint32_t* n_contrib, const float* dL_dcolor,
                            const float* dL_ddepth, const float* dL_dalpha, double* g10, double* g10abs) {
  const int gx = (s->W + TILE - 1) / TILE, gy = (s->H + TILE - 1) / TILE;
  const size_t HW = (size_t)s->W * s->H;
  const int64_t K = ranges[gx * gy];
  double* part = (double*)calloc((size_t)(K > 0 ? K : 1) * 10, sizeof(double));
  double* pabs = g10abs ? (double*)calloc((size_t)(K > 0 ? K : 1) * 20, sizeof(double)) : NULL;
#pragma omp parallel for schedule(dynamic, 4)
  for (int tile = 0; tile < gx * gy; ++tile) {
    const int tx = tile % gx, ty = tile / gx;
    for (int ly = 0; ly < TILE; ++ly)
      for (int lx = 0; lx < TILE; ++lx) {
        int px = tx * TILE + lx, py = ty * TILE + ly;
        if (px >= s->W || py >= s->H) continue;
        size_t pix = (size_t)py * s->W + px;
        float pxf = (float)px, pyf = (float)py;
        const double Tf = final_T[pix];
        const double dC[3] = {dL_dcolor[pix], dL_dcolor[HW + pix], dL_dcolor[2 * HW + pix]};
        const double dD = dL_ddepth ? dL_ddepth[pix] : 0.0;
        const double dA = dL_dalpha ? dL_dalpha[pix] : 0.0;
        const double bg_dot = s->bg[0] * dC[0] + s->bg[1] * dC[1] + s->bg[2] * dC[2];
        double T = Tf;
        double acc[4] = {0, 0, 0, 0}, lastc[4] = {0, 0, 0, 0}, last_a = 0.0;
        double unwound = 0.0; /* contributions of this pixel already unwound (back to front) */
        uint32_t last = n_contrib[pix];
        for (int64_t c = (int64_t)last - 1; c >= 0; --c) {
          uint32_t i = ranges[tile] + (uint32_t)c;
          uint32_t g = gid[i];
          float ca = -0.5f * o->conic_op[4 * g + 0];
          float cb = -o->conic_op[4 * g + 1];
          float cc = -0.5f * o->conic_op[4 * g + 2];
          float op = o->conic_op[4 * g + 3];
          float dxf = o->xy[2 * g] - pxf, dyf = o->xy[2 * g + 1] - pyf;
          float e = cb * (dxf * dyf);
          e = fmaf(cc * dyf, dyf, e);
          float power = fmaf(ca * dxf, dxf, e);
          if (power > 0.0f) continue;
          float Gf = oracle_exp(power);
          float alphaf = fminf(ALPHA_MAX, op * Gf);
          if (alphaf < ALPHA_MIN) continue;
          double G = Gf, alpha = alphaf, dx = dxf, dy = dyf;
          T = T / (1.0 - alpha);
          double w = alpha * T;
          double col[4] = {o->rgbd[4 * g], o->rgbd[4 * g + 1], o->rgbd[4 * g + 2], o->rgbd[4 * g + 3]};
          double* pp = part + (size_t)i * 10;
          double* pa = pabs ? pabs + (size_t)i * 20 : NULL;
          pp[6] += dC[0] * w;
          pp[7] += dC[1] * w;
          pp[8] += dC[2] * w;
          pp[9] += dD * w;
          double dLda = 0.0;
          for (int k = 0; k < 4; ++k) {
            acc[k] = last_a * lastc[k] + (1.0 - last_a) * acc[k];
            lastc[k] = col[k];
          }
          dLda = (col[0] - acc[0]) * dC[0] + (col[1] - acc[1]) * dC[1] + (col[2] - acc[2]) * dC[2] +
                 (col[3] - acc[3]) * dD;
          dLda *= T;
          last_a = alpha;
          dLda += Tf / (1.0 - alpha) * (dA - bg_dot);
          pp[5] += G * dLda;
          double dp = G * (op * dLda);
          pp[0] += dp * (2.0 * ca * dx + cb * dy);
          pp[1] += dp * (2.0 * cc * dy + cb * dx);
          pp[2] += -0.5 * dx * dx * dp;
          pp[3] += -dx * dy * dp;
          pp[4] += -0.5 * dy * dy * dp;
          if (pa) {
            /* Magnitudes of what each sum adds up: the same terms with every product and
               sum of products taken in absolute value (pa[0..9]), and the same weighted by
               the number of contributions of the pixel unwound before this one
               (pa[10..19]). A float32 evaluation of the sums, in any order, rounds on the
               scale of the first; the transmittance and the colour behind, rebuilt back to
               front one contribution at a time, carry a rounding per step, on the scale
               of the second. */
            const double adLda = (fabs(col[0]) + fabs(acc[0])) * fabs(dC[0]) + (fabs(col[1]) + fabs(acc[1])) * fabs(dC[1]) +
                                 (fabs(col[2]) + fabs(acc[2])) * fabs(dC[2]) + (fabs(col[3]) + fabs(acc[3])) * fabs(dD);
            const double aL = adLda * T + Tf / (1.0 - alpha) * (fabs(dA) + fabs(bg_dot));
            const double adp = G * op * aL;
            double t10[10];
            t10[0] = adp * (2.0 * fabs(ca * dx) + fabs(cb * dy));
            t10[1] = adp * (2.0 * fabs(cc * dy) + fabs(cb * dx));
            t10[2] = 0.5 * dx * dx * adp;
            t10[3] = fabs(dx * dy) * adp;
            t10[4] = 0.5 * dy * dy * adp;
            t10[5] = G * aL;
            t10[6] = fabs(dC[0]) * w;
            t10[7] = fabs(dC[1]) * w;
            t10[8] = fabs(dC[2]) * w;
            t10[9] = fabs(dD) * w;
            for (int k = 0; k < 10; ++k) {
              pa[k] += t10[k];
              pa[10 + k] += unwound * t10[k];
            }
          }
          unwound += 1.0;
        }
      }
  }
  memset(g10, 0, sizeof(double) * 10 * (size_t)N);
  for (int64_t i = 0; i < K; ++i)
    for (int k = 0; k < 10; ++k) g10[(size_t)gid[i] * 10 + k] += part[(size_t)i * 10 + k];
  if (pabs) {
    memset(g10abs, 0, sizeof(double) * 20 * (size_t)N);
    for (int64_t i = 0; i < K; ++i)
      for (int k = 0; k < 20; ++k) g10abs[(size_t)gid[i] * 20 + k] += pabs[(size_t)i * 20 + k];
    free(pabs);
  }
  free(part);
}

/* Preprocess backward in double from the per-Gaussian render gradients g10.
 * Outputs (float): dmeans2D [N,3], dcolors [N,3], dopacity [N], dmeans3D [N,3],
 * dcov3D [N,6], dsh [N,M,3] (if shs), dscales [N,3], drots [N,4] (if not cov3D). */
void oracle_preprocess_backward(const OSettings* s, const OGauss* g, const OGeom* o, const double* g10,
                                float* dmeans2D, float* dcolors, float* dopacity, float* dmeans3D, float* dcov3D,
                                float* dsh, float* dscales, float* drots) {
  const double W = s->W, H = s->H;
  const double fx = (float)s->W / (2.0f * s->tanfovx);
  const double fy = (float)s->H / (2.0f * s->tanfovy);
  const float* Vf = s->view;
  const float* Pf = s->proj;
  double V[16], P[16];
  for (int k = 0; k < 16; ++k) {
    V[k] = Vf[k];
    P[k] = Pf[k];
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < g->N; ++i) {
    const int M = g->M;
    for (int k = 0; k < 3; ++k) {
      dmeans2D[3 * i + k] = 0.f;
      dcolors[3 * i + k] = 0.f;
      dmeans3D[3 * i + k] = 0.f;
      if (dscales) dscales[3 * i + k] = 0.f;
    }
    dopacity[i] = 0.f;
    for (int k = 0; k < 6; ++k) dcov3D[6 * i + k] = 0.f;
    if (drots)
      for (int k = 0; k < 4; ++k) drots[4 * i + k] = 0.f;
    if (dsh)
      for (int k = 0; k < 3 * M; ++k) dsh[(size_t)i * 3 * M + k] = 0.f;
    if (o->radii[i] <= 0) continue;
    const double* a = g10 + (size_t)i * 10;
    const double dndc_x = a[0] * 0.5 * W, dndc_y = a[1] * 0.5 * H;
    dmeans2D[3 * i + 0] = (float)dndc_x;
    dmeans2D[3 * i + 1] = (float)dndc_y;
    dopacity[i] = (float)a[5];
    const double dcol[3] = {a[6], a[7], a[8]};
    for (int k = 0; k < 3; ++k) dcolors[3 * i + k] = (float)dcol[k];
    const double p[3] = {g->means3D[3 * i], g->means3D[3 * i + 1], g->means3D[3 * i + 2]};
    double t[3];
    for (int r = 0; r < 3; ++r) t[r] = V[r] * p[0] + V[4 + r] * p[1] + V[8 + r] * p[2] + V[12 + r];
    double cov[6], R[9] = {0}, sc[3] = {0}, q[4] = {0};
    const double mod = s->scale_modifier;
    if (g->cov3D) {
      for (int k = 0; k < 6; ++k) cov[k] = g->cov3D[6 * i + k];
    } else {
      for (int k = 0; k < 3; ++k) sc[k] = mod * g->scales[3 * i + k];
      for (int k = 0; k < 4; ++k) q[k] = g->rots[4 * i + k];
      double r = q[0], x = q[1], y = q[2], z = q[3];
      R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - r * z); R[2] = 2 * (x * z + r * y);
      R[3] = 2 * (x * y + r * z); R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - r * x);
      R[6] = 2 * (x * z - r * y); R[7] = 2 * (y * z + r * x); R[8] = 1 - 2 * (x * x + y * y);
      double Mm[9];
      for (int r2 = 0; r2 < 3; ++r2)
        for (int c = 0; c < 3; ++c) Mm[3 * r2 + c] = R[3 * r2 + c] * sc[c];
      static const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
      for (int k = 0; k < 6; ++k)
        cov[k] = Mm[3 * ii[k]] * Mm[3 * jj[k]] + Mm[3 * ii[k] + 1] * Mm[3 * jj[k] + 1] +
                 Mm[3 * ii[k] + 2] * Mm[3 * jj[k] + 2];
    }
    const double limx = 1.3 * (double)s->tanfovx, limy = 1.3 * (double)s->tanfovy;
    const double txtz = t[0] / t[2], tytz = t[1] / t[2];
    const double tx = fmin(limx, fmax(-limx, txtz)) * t[2];
    const double ty = fmin(limy, fmax(-limy, tytz)) * t[2];
    const double xm = (txtz < -limx || txtz > limx) ? 0.0 : 1.0;
    const double ym = (tytz < -limy || tytz > limy) ? 0.0 : 1.0;
    const double tz = t[2], tz2 = tz * tz, tz3 = tz2 * tz;
    const double J00 = fx / tz, J02 = -(fx * tx) / tz2, J11 = fy / tz, J12 = -(fy * ty) / tz2;
    double T0[3], T1[3];
    for (int j = 0; j < 3; ++j) {
      T0[j] = J00 * V[4 * j] + J02 * V[4 * j + 2];
      T1[j] = J11 * V[4 * j + 1] + J12 * V[4 * j + 2];
    }
    const double S[9] = {cov[0], cov[1], cov[2], cov[1], cov[3], cov[4], cov[2], cov[4], cov[5]};
    double u[3], v[3];
    for (int r = 0; r < 3; ++r) {
      u[r] = S[3 * r] * T0[0] + S[3 * r + 1] * T0[1] + S[3 * r + 2] * T0[2];
      v[r] = S[3 * r] * T1[0] + S[3 * r + 1] * T1[1] + S[3 * r + 2] * T1[2];
    }
    const double ca = T0[0] * u[0] + T0[1] * u[1] + T0[2] * u[2] + 0.3;
    const double cb = T0[0] * v[0] + T0[1] * v[1] + T0[2] * v[2];
    const double cc = T1[0] * v[0] + T1[1] * v[1] + T1[2] * v[2] + 0.3;
    const double dA = a[2], dB = a[3], dC = a[4];
    const double det = ca * cc - cb * cb, id = 1.0 / det, id2 = id * id;
    const double da = dA * (-cc * cc * id2) + dB * (cb * cc * id2) + dC * (-cb * cb * id2);
    const double db = dA * (2 * cb * cc * id2) + dB * (-id - 2 * cb * cb * id2) + dC * (2 * ca * cb * id2);
    const double dc = dA * (-cb * cb * id2) + dB * (ca * cb * id2) + dC * (-ca * ca * id2);
    double dcov[6];
    dcov[0] = da * T0[0] * T0[0] + db * T0[0] * T1[0] + dc * T1[0] * T1[0];
    dcov[3] = da * T0[1] * T0[1] + db * T0[1] * T1[1] + dc * T1[1] * T1[1];
    dcov[5] = da * T0[2] * T0[2] + db * T0[2] * T1[2] + dc * T1[2] * T1[2];
    dcov[1] = 2 * da * T0[0] * T0[1] + db * (T0[0] * T1[1] + T0[1] * T1[0]) + 2 * dc * T1[0] * T1[1];
    dcov[2] = 2 * da * T0[0] * T0[2] + db * (T0[0] * T1[2] + T0[2] * T1[0]) + 2 * dc * T1[0] * T1[2];
    dcov[4] = 2 * da * T0[1] * T0[2] + db * (T0[1] * T1[2] + T0[2] * T1[1]) + 2 * dc * T1[1] * T1[2];
    for (int k = 0; k < 6; ++k) dcov3D[6 * i + k] = (float)dcov[k];
    double dT0[3], dT1[3];
    for (int r = 0; r < 3; ++r) {
      dT0[r] = 2 * da * u[r] + db * v[r];
      dT1[r] = db * u[r] + 2 * dc * v[r];
    }
    double dJ00 = 0, dJ02 = 0, dJ11 = 0, dJ12 = 0;
    for (int j = 0; j < 3; ++j) {
      dJ00 += dT0[j] * V[4 * j];
      dJ02 += dT0[j] * V[4 * j + 2];
      dJ11 += dT1[j] * V[4 * j + 1];
      dJ12 += dT1[j] * V[4 * j + 2];
    }
    double dt[3];
    dt[0] = xm * dJ02 * (-fx / tz2);
    dt[1] = ym * dJ12 * (-fy / tz2);
    dt[2] = dJ00 * (-fx / tz2) + dJ11 * (-fy / tz2) + dJ02 * (2 * fx * tx / tz3) + dJ12 * (2 * fy * ty / tz3) + a[9];
    double dm[3];
    for (int j = 0; j < 3; ++j) dm[j] = V[4 * j] * dt[0] + V[4 * j + 1] * dt[1] + V[4 * j + 2] * dt[2];
    const double hx = P[0] * p[0] + P[4] * p[1] + P[8] * p[2] + P[12];
    const double hy = P[1] * p[0] + P[5] * p[1] + P[9] * p[2] + P[13];
    const double hw = P[3] * p[0] + P[7] * p[1] + P[11] * p[2] + P[15];
    const double wi = 1.0 / (hw + 1e-7), wi2 = wi * wi;
    for (int j = 0; j < 3; ++j)
      dm[j] += dndc_x * (P[4 * j] * wi - hx * wi2 * P[4 * j + 3]) + dndc_y * (P[4 * j + 1] * wi - hy * wi2 * P[4 * j + 3]);
    if (g->shs) {
      const uint8_t cl = o->clamped[i];
      const double gc[3] = {(cl & 1) ? 0.0 : dcol[0], (cl & 2) ? 0.0 : dcol[1], (cl & 4) ? 0.0 : dcol[2]};
      const float* sh = g->shs + (size_t)i * 3 * M;
      const double ddx = p[0] - s->campos[0], ddy = p[1] - s->campos[1], ddz = p[2] - s->campos[2];
      const double len = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
      const double x = ddx / len, y = ddy / len, z = ddz / len;
      /* basis values and their partial derivatives along x, y, z */
      double b[16] = {0}, bx[16] = {0}, by[16] = {0}, bz[16] = {0};
      const double c1 = SH_C1;
      const double c2[5] = {SH_C2[0], SH_C2[1], SH_C2[2], SH_C2[3], SH_C2[4]};
      const double c3[7] = {SH_C3[0], SH_C3[1], SH_C3[2], SH_C3[3], SH_C3[4], SH_C3[5], SH_C3[6]};
      const int deg = s->sh_degree;
      int nb = 1;
      b[0] = SH_C0;
      if (deg > 0) {
        b[1] = -c1 * y; by[1] = -c1;
        b[2] = c1 * z; bz[2] = c1;
        b[3] = -c1 * x; bx[3] = -c1;
        nb = 4;
      }
      if (deg > 1) {
        double xx = x * x, yy = y * y, zz = z * z;
        b[4] = c2[0] * x * y; bx[4] = c2[0] * y; by[4] = c2[0] * x;
        b[5] = c2[1] * y * z; by[5] = c2[1] * z; bz[5] = c2[1] * y;
        b[6] = c2[2] * (2 * zz - xx - yy); bx[6] = -2 * c2[2] * x; by[6] = -2 * c2[2] * y; bz[6] = 4 * c2[2] * z;
        b[7] = c2[3] * x * z; bx[7] = c2[3] * z; bz[7] = c2[3] * x;
        b[8] = c2[4] * (xx - yy); bx[8] = 2 * c2[4] * x; by[8] = -2 * c2[4] * y;
        nb = 9;
        if (deg > 2) {
          b[9] = c3[0] * y * (3 * xx - yy); bx[9] = c3[0] * 6 * x * y; by[9] = c3[0] * (3 * xx - 3 * yy);
          b[10] = c3[1] * x * y * z; bx[10] = c3[1] * y * z; by[10] = c3[1] * x * z; bz[10] = c3[1] * x * y;
          b[11] = c3[2] * y * (4 * zz - xx - yy); bx[11] = -2 * c3[2] * x * y;
          by[11] = c3[2] * (4 * zz - xx - 3 * yy); bz[11] = 8 * c3[2] * y * z;
          b[12] = c3[3] * z * (2 * zz - 3 * xx - 3 * yy); bx[12] = -6 * c3[3] * x * z; by[12] = -6 * c3[3] * y * z;
          bz[12] = c3[3] * (6 * zz - 3 * xx - 3 * yy);
          b[13] = c3[4] * x * (4 * zz - xx - yy); bx[13] = c3[4] * (4 * zz - 3 * xx - yy);
          by[13] = -2 * c3[4] * x * y; bz[13] = 8 * c3[4] * x * z;
          b[14] = c3[5] * z * (xx - yy); bx[14] = 2 * c3[5] * x * z; by[14] = -2 * c3[5] * y * z;
          bz[14] = c3[5] * (xx - yy);
          b[15] = c3[6] * x * (xx - 3 * yy); bx[15] = c3[6] * (3 * xx - 3 * yy); by[15] = -6 * c3[6] * x * y;
          nb = 16;
        }
      }
      double gdx = 0, gdy = 0, gdz = 0;
      for (int k = 0; k < nb && k < M; ++k) {
        if (dsh)
          for (int ch = 0; ch < 3; ++ch) dsh[(size_t)i * 3 * M + 3 * k + ch] = (float)(b[k] * gc[ch]);
        double sdot = sh[3 * k] * gc[0] + sh[3 * k + 1] * gc[1] + sh[3 * k + 2] * gc[2];
        gdx += sdot * bx[k];
        gdy += sdot * by[k];
        gdz += sdot * bz[k];
      }
      double dotv = x * gdx + y * gdy + z * gdz;
      dm[0] += (gdx - x * dotv) / len;
      dm[1] += (gdy - y * dotv) / len;
      dm[2] += (gdz - z * dotv) / len;
    }
    for (int j = 0; j < 3; ++j) dmeans3D[3 * i + j] = (float)dm[j];
    if (!g->cov3D) {
      double Mm[9];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Mm[3 * r + c] = R[3 * r + c] * sc[c];
      const double G[9] = {dcov[0], 0.5 * dcov[1], 0.5 * dcov[2], 0.5 * dcov[1], dcov[3],
                           0.5 * dcov[4], 0.5 * dcov[2], 0.5 * dcov[4], dcov[5]};
      double dM[9], dR[9];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          dM[3 * r + c] = 2 * (G[3 * r] * Mm[c] + G[3 * r + 1] * Mm[3 + c] + G[3 * r + 2] * Mm[6 + c]);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) dR[3 * r + c] = dM[3 * r + c] * sc[c];
      for (int c = 0; c < 3; ++c)
        dscales[3 * i + c] = (float)((dM[c] * R[c] + dM[3 + c] * R[3 + c] + dM[6 + c] * R[6 + c]) * mod);
      const double r = q[0], x = q[1], y = q[2], z = q[3];
      drots[4 * i + 0] = (float)(2 * (-z * dR[1] + y * dR[2] + z * dR[3] - x * dR[5] - y * dR[6] + x * dR[7]));
      drots[4 * i + 1] = (float)(2 * (y * dR[1] + z * dR[2] + y * dR[3] - 2 * x * dR[4] - r * dR[5] + z * dR[6] +
                                      r * dR[7] - 2 * x * dR[8]));
      drots[4 * i + 2] = (float)(2 * (-2 * y * dR[0] + x * dR[1] + r * dR[2] + x * dR[3] + z * dR[5] - r * dR[6] +
                                      z * dR[7] - 2 * y * dR[8]));
      drots[4 * i + 3] = (float)(2 * (-2 * z * dR[0] - r * dR[1] + x * dR[2] + r * dR[3] - 2 * z * dR[4] + y * dR[5] +
                                      x * dR[6] + y * dR[7]));
    }
  }
}
