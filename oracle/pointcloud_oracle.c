/*
 * CPU oracle of the frame-initialisation steps — TEST INFRASTRUCTURE ONLY (loaded by
 * tests/ and the smoke check as the checker, never by the product path).
 *
 * Restates, in the published algorithms' own form:
 *   - kornia depth_to_3d(normalize_points=False) as called at trainer/trainer.py:491:
 *     pixel (u, v) at depth d -> ((u - cx) / fx * d, (v - cy) / fy * d, d), float32;
 *   - Open3D PointCloud::VoxelDownSample as called at trainer/trainer.py:507: voxel
 *     index floor((p - (min - s/2)) / s) in double, points and colours of a voxel
 *     accumulated in double in input order and averaged; voxels listed here in
 *     increasing linear index ((ix ny + iy) nz + iz) order;
 *   - simple-knn distCUDA2 as called at scene/gaussian_model_cf.py:194: per point the
 *     mean of the squared distances to its three nearest other points, by brute force.
 * kornia, Open3D and simple-knn are unpinned dependencies (requirements.txt,
 * .gitmodules:1-3). Squared distances use the same rounding sequence as the kernels:
 * fmaf(dz, dz, fmaf(dy, dy, dx * dx)). Compiled with -ffp-contract=off.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

void oracle_depth_to_points(int H, int W, const float* depth, float fx, float fy, float cx, float cy, float* xyz) {
  for (int64_t i = 0; i < (int64_t)H * W; ++i) {
    const int u = (int)(i % W), v = (int)(i / W);
    const float d = depth[i];
    xyz[3 * i + 0] = (((float)u - cx) / fx) * d;
    xyz[3 * i + 1] = (((float)v - cy) / fy) * d;
    xyz[3 * i + 2] = d;
  }
}

static float dist2_ref(const float* a, const float* b) {
  const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

void oracle_knn3_mean_dist2(int64_t n, const float* xyz, float* out) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    float b0 = FLT_MAX, b1 = FLT_MAX, b2 = FLT_MAX;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i) continue;
      const float d = dist2_ref(xyz + 3 * i, xyz + 3 * j);
      if (d < b2) {
        if (d < b1) {
          b2 = b1;
          if (d < b0) {
            b1 = b0;
            b0 = d;
          } else {
            b1 = d;
          }
        } else {
          b2 = d;
        }
      }
    }
    out[i] = ((b0 + b1) + b2) / 3.0f;
  }
}

typedef struct {
  uint64_t key;
  int64_t idx;
} KeyIdx;

static int cmp_key_idx(const void* a, const void* b) {
  const KeyIdx* x = (const KeyIdx*)a;
  const KeyIdx* y = (const KeyIdx*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx ? 1 : 0);
}

/* Returns the number of voxels (out_* need room for n), or -1 if the grid is too large. */
int64_t oracle_voxel_down_sample(int64_t n, const float* xyz, const float* rgb, double s, float* out_xyz,
                                 float* out_rgb) {
  if (n <= 0) return 0;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int64_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      if (xyz[3 * i + a] < lo[a]) lo[a] = xyz[3 * i + a];
      if (xyz[3 * i + a] > hi[a]) hi[a] = xyz[3 * i + a];
    }
  double mn[3];
  uint64_t dim[3];
  for (int a = 0; a < 3; ++a) {
    mn[a] = (double)lo[a] - 0.5 * s;
    dim[a] = (uint64_t)floor(((double)hi[a] - mn[a]) / s) + 1;
  }
  KeyIdx* ki = (KeyIdx*)malloc(sizeof(KeyIdx) * (size_t)n);
  if (!ki) return -1;
  for (int64_t i = 0; i < n; ++i) {
    const double rx = ((double)xyz[3 * i + 0] - mn[0]) / s;
    const double ry = ((double)xyz[3 * i + 1] - mn[1]) / s;
    const double rz = ((double)xyz[3 * i + 2] - mn[2]) / s;
    ki[i].key = ((uint64_t)floor(rx) * dim[1] + (uint64_t)floor(ry)) * dim[2] + (uint64_t)floor(rz);
    ki[i].idx = i;
  }
  qsort(ki, (size_t)n, sizeof(KeyIdx), cmp_key_idx);
  int64_t m = 0;
  for (int64_t b = 0; b < n;) {
    int64_t e = b;
    double sum[6] = {0, 0, 0, 0, 0, 0};
    while (e < n && ki[e].key == ki[b].key) {
      const int64_t i = ki[e].idx;
      for (int a = 0; a < 3; ++a) sum[a] += (double)xyz[3 * i + a];
      if (rgb)
        for (int a = 0; a < 3; ++a) sum[3 + a] += (double)rgb[3 * i + a];
      ++e;
    }
    const double c = (double)(e - b);
    for (int a = 0; a < 3; ++a) out_xyz[3 * m + a] = (float)(sum[a] / c);
    if (rgb && out_rgb)
      for (int a = 0; a < 3; ++a) out_rgb[3 * m + a] = (float)(sum[3 + a] / c);
    ++m;
    b = e;
  }
  free(ki);
  return m;
}
