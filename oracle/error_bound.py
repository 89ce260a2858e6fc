"""Float32 rounding-error bound of the rasteriser backward — TEST INFRASTRUCTURE ONLY.

Only tests/ use this module. The C oracle (cfgs_oracle.c) forms every gradient in
float64; the CUDA kernels form the same quantities in float32, in another order. Where an
element's terms cancel, the two legitimately differ by more than a relative tolerance can
express. This module bounds that difference element by element with first-order running
error analysis (Higham, "Accuracy and Stability of Numerical Algorithms", 2nd ed., ch. 3):
every quantity x of the float32 computation carries a bound e(x) on |fl(x) - x|, and each
IEEE operation (u = 2^-24, round to nearest) propagates it:

    x + y : e = e(x) + e(y) + u |x + y|
    x * y : e = |x| e(y) + |y| e(x) + e(x) e(y) + u |x y|
    x / y : e = (e(x) + |x / y| e(y)) / (|y| - e(y)) + u |x / y|
    sqrt x: e = e(x) / (2 sqrt x) + u sqrt x

Inputs read from float32 arrays are exact (e = 0). The ten per-Gaussian 2D gradient sums
that enter the per-Gaussian chain carry the bound of the render backward's sums, from the
oracle's magnitudes of the summed terms (Oracle.backward(..., magnitudes=True)):

    e(sum_k) = u ((C_SUM + touched / 8) S_k + C_UNWIND W_k)

with S_k the sum of the terms' magnitudes and W_k the same weighted by the number of
contributions the pixel had unwound before (the back-to-front recursion rounds once or
twice per step: transmittance by an approximate reciprocal and a product, the colour
behind by a fused multiply-add). C_SUM covers the roundings of one term and of the tree
sums over a warp's 64 pixels, the 4 warps of a tile and a Gaussian's records.

The per-Gaussian chain below restates, operation for operation, the CUDA kernel's
conic -> 2D covariance -> 3D covariance -> scale/rotation, projection and SH chain (the
published 3DGS backward; the Python math it mirrors is utils/general_utils.py:76-108,
utils/sh_utils.py:57-112, scene/cameras.py:57-74), evaluated on these bounded numbers.
"""
from __future__ import annotations

import numpy as np

U = 2.0 ** -24
C_SUM = 24.0
C_UNWIND = 8.0

SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = [1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396]
SH_C3 = [-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154, -0.4570457994644658,
         1.445305721320277, -0.5900435899266435]


class B:
    """A float32 quantity: value (float64 numpy array) and a bound on its rounding error."""
    __slots__ = ("v", "e")

    def __init__(self, v, e=0.0):
        self.v = np.asarray(v, np.float64)
        self.e = np.broadcast_to(np.asarray(e, np.float64), self.v.shape)

    @staticmethod
    def of(x):
        return x if isinstance(x, B) else B(x, 0.0)

    def __add__(self, o):
        o = B.of(o)
        r = self.v + o.v
        return B(r, self.e + o.e + U * np.abs(r))

    __radd__ = __add__

    def __sub__(self, o):
        o = B.of(o)
        r = self.v - o.v
        return B(r, self.e + o.e + U * np.abs(r))

    def __rsub__(self, o):
        return B.of(o) - self

    def __neg__(self):
        return B(-self.v, self.e)

    def __mul__(self, o):
        o = B.of(o)
        r = self.v * o.v
        return B(r, np.abs(self.v) * o.e + np.abs(o.v) * self.e + self.e * o.e + U * np.abs(r))

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = B.of(o)
        with np.errstate(divide="ignore", invalid="ignore"):
            q = self.v / o.v
            den = np.abs(o.v) - o.e
            e = np.where(den > 0, (self.e + np.abs(q) * o.e) / np.where(den > 0, den, 1.0), np.inf) + U * np.abs(q)
        return B(q, e)

    def __rtruediv__(self, o):
        return B.of(o) / self

    def sqrt(self):
        r = np.sqrt(self.v)
        with np.errstate(divide="ignore", invalid="ignore"):
            e = np.where(r > 0, self.e / (2.0 * np.where(r > 0, r, 1.0)), np.sqrt(self.e)) + U * r
        return B(r, e)

    def masked(self, m):
        """The quantity where m holds, an exact zero elsewhere (a select, no rounding)."""
        return B(np.where(m, self.v, 0.0), np.where(m, self.e, 0.0))


def _dot3(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def contribution_counts(o) -> np.ndarray:
    """Per Gaussian, the number of (pixel, instance) pairs of the oracle's forward `o`
    that the backward visits: instance positions below the pixel's contributor count.
    An upper bound on the terms one Gaussian's gradient sums add up."""
    out = np.zeros(o.N, np.float64)
    nc = o.n_contrib.reshape(o.H, o.W)
    for t in range(o.gx * o.gy):
        tx, ty = t % o.gx, t // o.gx
        blk = nc[ty * 16:(ty + 1) * 16, tx * 16:(tx + 1) * 16].ravel().astype(np.int64)
        m = int(blk.max()) if blk.size else 0
        if m == 0:
            continue
        at_least = np.cumsum(np.bincount(blk, minlength=m + 1)[::-1])[::-1]  # pixels with count >= v
        lo = int(o.ranges[t])
        np.add.at(out, o.gid[lo:lo + m].astype(np.int64), at_least[1:m + 1].astype(np.float64))
    return out


def backward_bounds(o, terms=None) -> dict:
    """Per output element, a bound on the float32 rounding error of the kernels'
    gradients for the oracle `o` after o.backward(..., magnitudes=True). Returns arrays
    shaped like the outputs of Oracle.backward (None where that output is absent).

    `terms` (per Gaussian, e.g. contribution_counts(o)) replaces the tree-sum depth
    touched / 8 by the number of terms: the bound of a sum formed in any order, one term
    at a time (n terms in any order: at most (n - 1) u times the sum of magnitudes), as
    global atomic accumulation forms it."""
    if getattr(o, "g10abs", None) is None:
        raise RuntimeError("call Oracle.backward(..., magnitudes=True) first")
    k = o._keep
    N = o.N
    vis = o.radii > 0
    idx = np.nonzero(vis)[0]
    n = idx.size
    out = {"means2D": np.zeros((N, 3)), "colors": np.zeros((N, 3)), "opacity": np.zeros((N, 1)),
           "means3D": np.zeros((N, 3)), "cov3D": np.zeros((N, 6)),
           "sh": np.zeros((N, o.M, 3)) if k["shs"] is not None else None,
           "scales": np.zeros((N, 3)) if k["cov"] is None else None,
           "rotations": np.zeros((N, 4)) if k["cov"] is None else None}
    if n == 0:
        return out
    S = o.g10abs[idx, :10]
    Wt = o.g10abs[idx, 10:]
    spread = o.touched[idx].astype(np.float64) / 8.0 if terms is None else np.asarray(terms, np.float64)[idx]
    acc = [B(o.g10[idx, j], U * ((C_SUM + spread) * S[:, j] + C_UNWIND * Wt[:, j])) for j in range(10)]

    W, H = float(o.W), float(o.H)
    V = [float(x) for x in k["view"]]
    P = [float(x) for x in k["proj"]]
    p = k["means"][idx].astype(np.float64)
    px, py, pz = B(p[:, 0]), B(p[:, 1]), B(p[:, 2])
    f32 = lambda x: float(np.float32(x))
    dndc_x = acc[0] * (0.5 * W)
    dndc_y = acc[1] * (0.5 * H)
    out["means2D"][idx, 0] = dndc_x.e
    out["means2D"][idx, 1] = dndc_y.e
    out["opacity"][idx, 0] = acc[5].e
    for c in range(3):
        out["colors"][idx, c] = acc[6 + c].e

    t = [((px * V[i] + py * V[4 + i]) + pz * V[8 + i]) + V[12 + i] for i in range(3)]
    mod = f32(o.s.scale_modifier)
    if k["cov"] is not None:
        cv = k["cov"][idx].astype(np.float64)
        cov = [B(cv[:, j]) for j in range(6)]
    else:
        sc = k["scales"][idx].astype(np.float64)
        q = k["rots"][idx].astype(np.float64)
        s3 = [B(sc[:, j]) * mod for j in range(3)]
        qr, qx, qy, qz = (B(q[:, j]) for j in range(4))
        R = [1.0 - 2.0 * (qy * qy + qz * qz), 2.0 * (qx * qy - qr * qz), 2.0 * (qx * qz + qr * qy),
             2.0 * (qx * qy + qr * qz), 1.0 - 2.0 * (qx * qx + qz * qz), 2.0 * (qy * qz - qr * qx),
             2.0 * (qx * qz - qr * qy), 2.0 * (qy * qz + qr * qx), 1.0 - 2.0 * (qx * qx + qy * qy)]
        Mm = [R[3 * i + j] * s3[j] for i in range(3) for j in range(3)]
        ii, jj = [0, 0, 0, 1, 1, 2], [0, 1, 2, 1, 2, 2]
        cov = [_dot3(Mm[3 * ii[m]: 3 * ii[m] + 3], Mm[3 * jj[m]: 3 * jj[m] + 3]) for m in range(6)]
    tanx, tany = f32(o.s.tanfovx), f32(o.s.tanfovy)
    limx, limy = f32(np.float32(1.3) * np.float32(tanx)), f32(np.float32(1.3) * np.float32(tany))
    txtz, tytz = t[0] / t[2], t[1] / t[2]
    xm = ~((txtz.v < -limx) | (txtz.v > limx))
    ym = ~((tytz.v < -limy) | (tytz.v > limy))
    tx = B(np.clip(txtz.v, -limx, limx), np.where(xm, txtz.e, 0.0)) * t[2]
    ty = B(np.clip(tytz.v, -limy, limy), np.where(ym, tytz.e, 0.0)) * t[2]
    tz = t[2]
    tz2 = tz * tz
    tz3 = tz2 * tz
    fx = f32(np.float32(W) / (np.float32(2.0) * np.float32(tanx)))
    fy = f32(np.float32(H) / (np.float32(2.0) * np.float32(tany)))
    J00, J02 = fx / tz, -((tx * fx) / tz2)
    J11, J12 = fy / tz, -((ty * fy) / tz2)
    T0 = [J00 * V[4 * j] + J02 * V[4 * j + 2] for j in range(3)]
    T1 = [J11 * V[4 * j + 1] + J12 * V[4 * j + 2] for j in range(3)]
    Sm = [cov[0], cov[1], cov[2], cov[1], cov[3], cov[4], cov[2], cov[4], cov[5]]
    u = [_dot3(Sm[3 * i: 3 * i + 3], T0) for i in range(3)]
    v = [_dot3(Sm[3 * i: 3 * i + 3], T1) for i in range(3)]
    ca = _dot3(T0, u) + f32(0.3)
    cb = _dot3(T0, v)
    cc = _dot3(T1, v) + f32(0.3)
    dA, dB, dC = acc[2], acc[3], acc[4]
    det = ca * cc - cb * cb
    iD = 1.0 / det
    iD2 = iD * iD
    da = (dA * (-(cc * cc * iD2)) + dB * (cb * cc * iD2)) + dC * (-((cb * cb) * iD2))
    db = (dA * (2.0 * cb * cc * iD2) + dB * (-iD - 2.0 * cb * cb * iD2)) + dC * (2.0 * ca * cb * iD2)
    dc = (dA * (-((cb * cb) * iD2)) + dB * (ca * cb * iD2)) + dC * (-(ca * ca * iD2))
    dcov = [None] * 6
    for m, j in ((0, 0), (3, 1), (5, 2)):
        dcov[m] = (da * T0[j] * T0[j] + db * T0[j] * T1[j]) + dc * T1[j] * T1[j]
    for m, (a_, b_) in ((1, (0, 1)), (2, (0, 2)), (4, (1, 2))):
        dcov[m] = (2.0 * da * T0[a_] * T0[b_] + db * (T0[a_] * T1[b_] + T0[b_] * T1[a_])) + 2.0 * dc * T1[a_] * T1[b_]
    for m in range(6):
        out["cov3D"][idx, m] = dcov[m].e
    dT0 = [2.0 * da * u[i] + db * v[i] for i in range(3)]
    dT1 = [db * u[i] + 2.0 * dc * v[i] for i in range(3)]
    dJ00 = _dot3(dT0, [V[0], V[4], V[8]])
    dJ02 = _dot3(dT0, [V[2], V[6], V[10]])
    dJ11 = _dot3(dT1, [V[1], V[5], V[9]])
    dJ12 = _dot3(dT1, [V[2], V[6], V[10]])
    dt0 = (dJ02 * (-fx / tz2)).masked(xm)
    dt1 = (dJ12 * (-fy / tz2)).masked(ym)
    dt2 = (((dJ00 * (-fx / tz2) + dJ11 * (-fy / tz2)) + dJ02 * ((2.0 * fx) * tx / tz3)) +
           dJ12 * ((2.0 * fy) * ty / tz3)) + acc[9]
    dmean = [(V[4 * j] * dt0 + V[4 * j + 1] * dt1) + V[4 * j + 2] * dt2 for j in range(3)]
    hx = ((px * P[0] + py * P[4]) + pz * P[8]) + P[12]
    hy = ((px * P[1] + py * P[5]) + pz * P[9]) + P[13]
    hw = ((px * P[3] + py * P[7]) + pz * P[11]) + P[15]
    wi = 1.0 / (hw + f32(1e-7))
    wi2 = wi * wi
    for j in range(3):
        dmean[j] = dmean[j] + (dndc_x * (P[4 * j] * wi - hx * wi2 * P[4 * j + 3]) +
                               dndc_y * (P[4 * j + 1] * wi - hy * wi2 * P[4 * j + 3]))
    if k["shs"] is not None:
        M = o.M
        cl = o.clamped[idx]
        g = [acc[6 + c].masked((cl & (1 << c)) == 0) for c in range(3)]
        cp = [float(x) for x in k["campos"]]
        ddx, ddy, ddz = px - cp[0], py - cp[1], pz - cp[2]
        ln = ((ddx * ddx + ddy * ddy) + ddz * ddz).sqrt()
        x, y, z = ddx / ln, ddy / ln, ddz / ln
        deg = int(o.s.sh_degree)
        sh = k["shs"][idx].astype(np.float64)
        nb = (deg + 1) ** 2
        xx, yy, zz, xy, yz, xz = x * x, y * y, z * z, x * y, y * z, x * z
        b = [B(np.full(n, SH_C0))]
        if deg > 0:
            b += [-SH_C1 * y, SH_C1 * z, -SH_C1 * x]
        if deg > 1:
            b += [SH_C2[0] * xy, SH_C2[1] * yz, SH_C2[2] * (2.0 * zz - xx - yy), SH_C2[3] * xz, SH_C2[4] * (xx - yy)]
        if deg > 2:
            b += [SH_C3[0] * y * (3.0 * xx - yy), SH_C3[1] * xy * z, SH_C3[2] * y * (4.0 * zz - xx - yy),
                  SH_C3[3] * z * (2.0 * zz - 3.0 * xx - 3.0 * yy), SH_C3[4] * x * (4.0 * zz - xx - yy),
                  SH_C3[5] * z * (xx - yy), SH_C3[6] * x * (xx - 3.0 * yy)]
        sk = [(g[0] * sh[:, kk, 0] + g[1] * sh[:, kk, 1]) + g[2] * sh[:, kk, 2] for kk in range(min(nb, M))]
        zero = B(np.zeros(n))
        sk += [zero] * (16 - len(sk))
        gdx, gdy, gdz = zero, zero, zero
        if deg > 0:
            gdy = gdy - SH_C1 * sk[1]
            gdz = gdz + SH_C1 * sk[2]
            gdx = gdx - SH_C1 * sk[3]
        if deg > 1:
            gdx = gdx + (((SH_C2[0] * y * sk[4] - 2.0 * SH_C2[2] * x * sk[6]) + SH_C2[3] * z * sk[7]) +
                         2.0 * SH_C2[4] * x * sk[8])
            gdy = gdy + (((SH_C2[0] * x * sk[4] + SH_C2[1] * z * sk[5]) - 2.0 * SH_C2[2] * y * sk[6]) -
                         2.0 * SH_C2[4] * y * sk[8])
            gdz = gdz + ((SH_C2[1] * y * sk[5] + 4.0 * SH_C2[2] * z * sk[6]) + SH_C2[3] * x * sk[7])
        if deg > 2:
            gdx = gdx + ((((((SH_C3[0] * 6.0 * xy * sk[9] + SH_C3[1] * yz * sk[10]) - 2.0 * SH_C3[2] * xy * sk[11]) -
                            6.0 * SH_C3[3] * xz * sk[12]) + SH_C3[4] * (4.0 * zz - 3.0 * xx - yy) * sk[13]) +
                          2.0 * SH_C3[5] * xz * sk[14]) + SH_C3[6] * (3.0 * xx - 3.0 * yy) * sk[15])
            gdy = gdy + ((((((SH_C3[0] * (3.0 * xx - 3.0 * yy) * sk[9] + SH_C3[1] * xz * sk[10]) +
                             SH_C3[2] * (4.0 * zz - xx - 3.0 * yy) * sk[11]) - 6.0 * SH_C3[3] * yz * sk[12]) -
                           2.0 * SH_C3[4] * xy * sk[13]) - 2.0 * SH_C3[5] * yz * sk[14]) -
                         6.0 * SH_C3[6] * xy * sk[15])
            gdz = gdz + ((((SH_C3[1] * xy * sk[10] + 8.0 * SH_C3[2] * yz * sk[11]) +
                           SH_C3[3] * (6.0 * zz - 3.0 * xx - 3.0 * yy) * sk[12]) + 8.0 * SH_C3[4] * xz * sk[13]) +
                         SH_C3[5] * (xx - yy) * sk[14])
        for kk in range(M):
            for c in range(3):
                out["sh"][idx, kk, c] = (b[kk] * g[c]).e if kk < nb else 0.0
        dotv = (x * gdx + y * gdy) + z * gdz
        dmean[0] = dmean[0] + (gdx - x * dotv) / ln
        dmean[1] = dmean[1] + (gdy - y * dotv) / ln
        dmean[2] = dmean[2] + (gdz - z * dotv) / ln
    for j in range(3):
        out["means3D"][idx, j] = dmean[j].e
    if k["cov"] is None:
        G = [dcov[0], 0.5 * dcov[1], 0.5 * dcov[2], 0.5 * dcov[1], dcov[3], 0.5 * dcov[4], 0.5 * dcov[2],
             0.5 * dcov[4], dcov[5]]
        dM = [2.0 * ((G[3 * i] * Mm[j] + G[3 * i + 1] * Mm[3 + j]) + G[3 * i + 2] * Mm[6 + j])
              for i in range(3) for j in range(3)]
        dR = [dM[3 * i + j] * s3[j] for i in range(3) for j in range(3)]
        for j in range(3):
            out["scales"][idx, j] = (((dM[j] * R[j] + dM[3 + j] * R[3 + j]) + dM[6 + j] * R[6 + j]) * mod).e
        r, x_, y_, z_ = qr, qx, qy, qz
        dq = [2.0 * (((((-z_ * dR[1] + y_ * dR[2]) + z_ * dR[3]) - x_ * dR[5]) - y_ * dR[6]) + x_ * dR[7]),
              2.0 * (((((((y_ * dR[1] + z_ * dR[2]) + y_ * dR[3]) - 2.0 * x_ * dR[4]) - r * dR[5]) + z_ * dR[6]) +
                      r * dR[7]) - 2.0 * x_ * dR[8]),
              2.0 * (((((((-2.0 * y_ * dR[0] + x_ * dR[1]) + r * dR[2]) + x_ * dR[3]) + z_ * dR[5]) - r * dR[6]) +
                      z_ * dR[7]) - 2.0 * y_ * dR[8]),
              2.0 * (((((((-2.0 * z_ * dR[0] - r * dR[1]) + x_ * dR[2]) + r * dR[3]) - 2.0 * z_ * dR[4]) +
                       y_ * dR[5]) + x_ * dR[6]) + y_ * dR[7])]
        for j in range(4):
            out["rotations"][idx, j] = dq[j].e
    return out
