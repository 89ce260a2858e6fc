"""ctypes wrapper of the C oracle (oracle/cfgs_oracle.c) — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module,
as the checker. It works on host (numpy/torch-CPU) arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_u64p = C.POINTER(C.c_uint64)
_u8p = C.POINTER(C.c_uint8)


class OSettings(C.Structure):
    _fields_ = [("H", C.c_int), ("W", C.c_int), ("tanfovx", C.c_float), ("tanfovy", C.c_float), ("bg", _fp),
                ("scale_modifier", C.c_float), ("view", _fp), ("proj", _fp), ("sh_degree", C.c_int), ("campos", _fp)]


class OGauss(C.Structure):
    _fields_ = [("N", C.c_int), ("means3D", _fp), ("opac", _fp), ("shs", _fp), ("M", C.c_int), ("colors", _fp),
                ("scales", _fp), ("rots", _fp), ("cov3D", _fp)]


class OGeom(C.Structure):
    _fields_ = [("radii", _i32p), ("xy", _fp), ("conic_op", _fp), ("rgbd", _fp), ("rect", _i32p),
                ("touched", _u32p), ("clamped", _u8p)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(str(_build.build()))
        L.oracle_set_threads.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_exp.restype = C.c_float
        L.oracle_exp.argtypes = [C.c_float]
        L.oracle_preprocess.restype = C.c_int64
        L.oracle_preprocess.argtypes = [C.POINTER(OSettings), C.POINTER(OGauss), C.POINTER(OGeom)]
        L.oracle_bin.restype = None
        L.oracle_bin.argtypes = [C.POINTER(OSettings), C.c_int, C.POINTER(OGeom), C.c_int64, _u64p, _u32p, _u32p]
        L.oracle_render.restype = None
        L.oracle_render.argtypes = [C.POINTER(OSettings), C.POINTER(OGeom), _u32p, _u32p, _fp, _fp, _fp, _fp, _u32p]
        L.oracle_render_backward.restype = None
        L.oracle_render_backward.argtypes = [C.POINTER(OSettings), C.c_int, C.POINTER(OGeom), _u32p, _u32p, _fp,
                                             _u32p, _fp, _fp, _fp, _dp, _dp]
        L.oracle_preprocess_backward.restype = None
        L.oracle_preprocess_backward.argtypes = [C.POINTER(OSettings), C.POINTER(OGauss), C.POINTER(OGeom), _dp,
                                                 _fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp]
        _LIB = L
    return _LIB


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(int(n))


def exp(x: float) -> float:
    return lib().oracle_exp(float(x))


def _np(t, dtype=np.float32):
    if t is None:
        return None
    if hasattr(t, "detach"):
        t = t.detach().cpu().numpy()
    return np.ascontiguousarray(t, dtype=dtype)


def _p(a, ptype):
    return None if a is None else a.ctypes.data_as(ptype)


class Oracle:
    """One rasteriser call on the CPU: forward() then, optionally, backward()."""

    def __init__(self, width, height, tanfovx, tanfovy, bg, scale_modifier, viewmatrix, projmatrix, sh_degree,
                 campos, means3D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
                 cov3D_precomp=None):
        self.W, self.H = int(width), int(height)
        self._keep = {}
        k = self._keep
        k["bg"] = _np(bg).reshape(3)
        k["view"] = _np(viewmatrix).reshape(16)
        k["proj"] = _np(projmatrix).reshape(16)
        k["campos"] = _np(campos).reshape(3) if campos is not None else np.zeros(3, np.float32)
        k["means"] = _np(means3D).reshape(-1, 3)
        k["opac"] = _np(opacities).reshape(-1)
        self.N = k["means"].shape[0]
        k["shs"] = _np(shs)
        self.M = 0 if shs is None else int(k["shs"].shape[1])
        k["colors"] = _np(colors_precomp)
        k["scales"] = _np(scales)
        k["rots"] = _np(rotations)
        k["cov"] = _np(cov3D_precomp)
        self.s = OSettings(self.H, self.W, float(tanfovx), float(tanfovy), _p(k["bg"], _fp), float(scale_modifier),
                           _p(k["view"], _fp), _p(k["proj"], _fp), int(sh_degree), _p(k["campos"], _fp))
        self.g = OGauss(self.N, _p(k["means"], _fp), _p(k["opac"], _fp), _p(k["shs"], _fp), self.M,
                        _p(k["colors"], _fp), _p(k["scales"], _fp), _p(k["rots"], _fp), _p(k["cov"], _fp))
        self.gx = (self.W + 15) // 16
        self.gy = (self.H + 15) // 16

    @classmethod
    def from_scene(cls, scene, scale_modifier=1.0, bg=None, use_cov=False, use_colors=False, colors=None, cov=None):
        cam = scene.camera
        return cls(cam.width, cam.height, cam.tanfovx, cam.tanfovy, scene.bg if bg is None else bg, scale_modifier,
                   cam.viewmatrix, cam.projmatrix, scene.sh_degree, cam.campos, scene.means3D, scene.opacities,
                   shs=None if use_colors else scene.shs, colors_precomp=colors if use_colors else None,
                   scales=None if use_cov else scene.scales, rotations=None if use_cov else scene.rotations,
                   cov3D_precomp=cov if use_cov else None)

    def forward(self):
        L = lib()
        N = self.N
        self.radii = np.zeros(N, np.int32)
        self.xy = np.zeros((N, 2), np.float32)
        self.conic_op = np.zeros((N, 4), np.float32)
        self.rgbd = np.zeros((N, 4), np.float32)
        self.rect = np.zeros((N, 4), np.int32)
        self.touched = np.zeros(N, np.uint32)
        self.clamped = np.zeros(N, np.uint8)
        self.geom = OGeom(_p(self.radii, _i32p), _p(self.xy, _fp), _p(self.conic_op, _fp), _p(self.rgbd, _fp),
                          _p(self.rect, _i32p), _p(self.touched, _u32p), _p(self.clamped, _u8p))
        K = int(L.oracle_preprocess(C.byref(self.s), C.byref(self.g), C.byref(self.geom)))
        self.K = K
        self.keys = np.zeros(max(K, 1), np.uint64)
        self.gid = np.zeros(max(K, 1), np.uint32)
        self.ranges = np.zeros(self.gx * self.gy + 1, np.uint32)
        L.oracle_bin(C.byref(self.s), N, C.byref(self.geom), K, _p(self.keys, _u64p), _p(self.gid, _u32p),
                     _p(self.ranges, _u32p))
        HW = self.W * self.H
        self.color = np.zeros((3, self.H, self.W), np.float32)
        self.depth = np.zeros((1, self.H, self.W), np.float32)
        self.alpha = np.zeros((1, self.H, self.W), np.float32)
        self.final_T = np.zeros(HW, np.float32)
        self.n_contrib = np.zeros(HW, np.uint32)
        L.oracle_render(C.byref(self.s), C.byref(self.geom), _p(self.gid, _u32p), _p(self.ranges, _u32p),
                        _p(self.color, _fp), _p(self.depth, _fp), _p(self.alpha, _fp), _p(self.final_T, _fp),
                        _p(self.n_contrib, _u32p))
        self.keys = self.keys[:K]
        self.gid = self.gid[:K]
        return self

    def backward(self, dL_dcolor, dL_ddepth=None, dL_dalpha=None, magnitudes=False):
        """Gradients of every input (float64 sums rounded to float32 at the end). With
        magnitudes=True it also keeps, per Gaussian, the magnitudes of the per-pixel terms
        behind its ten 2D gradient sums (self.g10abs [N,20]: the sums of their absolute
        values, then the same weighted by the contributions unwound before each), which
        oracle.error_bound turns into per-element float32 rounding bounds."""
        L = lib()
        N, M = self.N, self.M
        dc = _np(dL_dcolor).reshape(-1)
        dd = _np(dL_ddepth).reshape(-1) if dL_ddepth is not None else None
        da = _np(dL_dalpha).reshape(-1) if dL_dalpha is not None else None
        g10 = np.zeros((max(N, 1), 10), np.float64)
        g10abs = np.zeros((max(N, 1), 20), np.float64) if magnitudes else None
        gid = self.gid if self.K > 0 else np.zeros(1, np.uint32)
        L.oracle_render_backward(C.byref(self.s), N, C.byref(self.geom), _p(gid, _u32p), _p(self.ranges, _u32p),
                                 _p(self.final_T, _fp), _p(self.n_contrib, _u32p), _p(dc, _fp), _p(dd, _fp),
                                 _p(da, _fp), _p(g10, _dp), _p(g10abs, _dp))
        self.g10 = g10[:N]
        self.g10abs = None if g10abs is None else g10abs[:N]
        return self._preprocess_backward(g10)

    def _preprocess_backward(self, g10):
        L = lib()
        N, M = self.N, self.M
        g10 = np.ascontiguousarray(g10, np.float64)
        out = {
            "means2D": np.zeros((N, 3), np.float32),
            "colors": np.zeros((N, 3), np.float32),
            "opacity": np.zeros((N, 1), np.float32),
            "means3D": np.zeros((N, 3), np.float32),
            "cov3D": np.zeros((N, 6), np.float32),
            "sh": np.zeros((N, M, 3), np.float32) if self._keep["shs"] is not None else None,
            "scales": np.zeros((N, 3), np.float32) if self._keep["cov"] is None else None,
            "rotations": np.zeros((N, 4), np.float32) if self._keep["cov"] is None else None,
        }
        L.oracle_preprocess_backward(C.byref(self.s), C.byref(self.g), C.byref(self.geom), _p(g10, _dp),
                                     _p(out["means2D"], _fp), _p(out["colors"], _fp), _p(out["opacity"], _fp),
                                     _p(out["means3D"], _fp), _p(out["cov3D"], _fp), _p(out["sh"], _fp),
                                     _p(out["scales"], _fp), _p(out["rotations"], _fp))
        return out


# ---- frame initialisation (oracle/pointcloud_oracle.c) ----------------------------------
def _pc_lib():
    L = lib()
    if not getattr(L, "_pc_ready", False):
        L.oracle_depth_to_points.restype = None
        L.oracle_depth_to_points.argtypes = [C.c_int, C.c_int, _fp, C.c_float, C.c_float, C.c_float, C.c_float, _fp]
        L.oracle_knn3_mean_dist2.restype = None
        L.oracle_knn3_mean_dist2.argtypes = [C.c_int64, _fp, _fp]
        L.oracle_voxel_down_sample.restype = C.c_int64
        L.oracle_voxel_down_sample.argtypes = [C.c_int64, _fp, _fp, C.c_double, _fp, _fp]
        L._pc_ready = True
    return L


def _f32c(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def depth_to_points(depth, fx, fy, cx, cy):
    d = _f32c(depth)
    H, W = d.shape
    out = np.empty((H * W, 3), np.float32)
    _pc_lib().oracle_depth_to_points(H, W, d.ctypes.data_as(_fp), fx, fy, cx, cy, out.ctypes.data_as(_fp))
    return out


def knn3_mean_dist2(points):
    p = _f32c(points).reshape(-1, 3)
    out = np.empty(p.shape[0], np.float32)
    _pc_lib().oracle_knn3_mean_dist2(p.shape[0], p.ctypes.data_as(_fp), out.ctypes.data_as(_fp))
    return out


def voxel_down_sample(points, colors, voxel_size):
    p = _f32c(points).reshape(-1, 3)
    c = None if colors is None else _f32c(colors).reshape(-1, 3)
    op = np.empty_like(p)
    oc = None if c is None else np.empty_like(c)
    m = _pc_lib().oracle_voxel_down_sample(p.shape[0], p.ctypes.data_as(_fp),
                                           None if c is None else c.ctypes.data_as(_fp), float(voxel_size),
                                           op.ctypes.data_as(_fp), None if oc is None else oc.ctypes.data_as(_fp))
    return op[:m], (None if oc is None else oc[:m])
