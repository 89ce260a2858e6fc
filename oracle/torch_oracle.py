"""Differentiable float64 restatement of the rasteriser in PyTorch (CPU) — TEST
INFRASTRUCTURE ONLY (used by tests/ to check gradients by autograd).

Independent of both the CUDA kernels and the C oracle: every discrete decision
(culling, radius, tile rectangle, depth order, skip and termination masks) is made here
in float64, and gradients come from autograd rather than hand derivation. Gradient
conventions of the published 3DGS rasteriser are reproduced explicitly:
- alpha = min(0.99, o G) passes gradient straight through the clamp;
- with the Jacobian clamp at 1.3 tan(fov), the clamped t.x (t.y) is treated as a
  constant (no gradient to t.x, none through t.x to t.z);
- means2D (a zero tensor in CF-3DGS, scene/gaussian_model_cf.py:793-801) enters as an
  additive offset of the NDC position, so its gradient is dL/dNDC.
The SH basis follows utils/sh_utils.py:57-112, the covariance
utils/general_utils.py:76-108, the matrices scene/cameras.py:57-74.
Dense per tile: meant for small scenes (hundreds to a few thousand Gaussians).
"""
from __future__ import annotations

import torch

SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = [1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396]
SH_C3 = [-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154, -0.4570457994644658,
         1.445305721320277, -0.5900435899266435]


def sh_basis(deg: int, d: torch.Tensor) -> torch.Tensor:
    """[N, (deg+1)^2] real SH basis values at unit directions d [N,3]."""
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    b = [torch.full_like(x, SH_C0)]
    if deg > 0:
        b += [-SH_C1 * y, SH_C1 * z, -SH_C1 * x]
    if deg > 1:
        xx, yy, zz = x * x, y * y, z * z
        b += [SH_C2[0] * x * y, SH_C2[1] * y * z, SH_C2[2] * (2 * zz - xx - yy), SH_C2[3] * x * z,
              SH_C2[4] * (xx - yy)]
        if deg > 2:
            b += [SH_C3[0] * y * (3 * xx - yy), SH_C3[1] * x * y * z, SH_C3[2] * y * (4 * zz - xx - yy),
                  SH_C3[3] * z * (2 * zz - 3 * xx - 3 * yy), SH_C3[4] * x * (4 * zz - xx - yy),
                  SH_C3[5] * z * (xx - yy), SH_C3[6] * x * (xx - 3 * yy)]
    return torch.stack(b, dim=1)


def rotation_matrix(q: torch.Tensor) -> torch.Tensor:
    """R from (r,x,y,z) without normalisation (the rasteriser's convention)."""
    r, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y),
        2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x),
        2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], dim=1).reshape(-1, 3, 3)


def cov3d(scales: torch.Tensor, rots: torch.Tensor, mod: float) -> torch.Tensor:
    R = rotation_matrix(rots)
    M = R * (mod * scales)[:, None, :]
    S = M @ M.transpose(1, 2)
    return torch.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], dim=1)


def rasterize(W, H, tanfovx, tanfovy, bg, scale_modifier, viewmatrix, projmatrix, sh_degree, campos, means3D,
              means2D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None, cov3D_precomp=None,
              tile=16):
    """Returns dict(color [3,H,W], depth [1,H,W], alpha [1,H,W], radii [N], n_contrib [H*W]).
    Differentiable (float64) w.r.t. every tensor argument that requires grad."""
    dt = torch.float64
    V = viewmatrix.to(dt)
    P = projmatrix.to(dt)
    p = means3D.to(dt)
    N = p.shape[0]
    ones = torch.ones(N, 1, dtype=dt)
    ph = torch.cat([p, ones], 1)
    t = ph @ V[:, :3]
    hom = ph @ P
    w_inv = 1.0 / (hom[:, 3] + 1e-7)
    ndc = hom[:, :2] * w_inv[:, None] + means2D.to(dt)[:, :2]
    pix_x = ((ndc[:, 0] + 1) * W - 1) * 0.5
    pix_y = ((ndc[:, 1] + 1) * H - 1) * 0.5
    if cov3D_precomp is not None:
        cov = cov3D_precomp.to(dt)
    else:
        cov = cov3d(scales.to(dt), rotations.to(dt), scale_modifier)
    fx = W / (2.0 * tanfovx)
    fy = H / (2.0 * tanfovy)
    limx, limy = 1.3 * tanfovx, 1.3 * tanfovy
    tz = t[:, 2]
    txtz, tytz = t[:, 0] / tz, t[:, 1] / tz
    inx = (txtz >= -limx) & (txtz <= limx)
    iny = (tytz >= -limy) & (tytz <= limy)
    tx = torch.where(inx, t[:, 0], (txtz.clamp(-limx, limx) * tz).detach())
    ty = torch.where(iny, t[:, 1], (tytz.clamp(-limy, limy) * tz).detach())
    J00, J02 = fx / tz, -fx * tx / (tz * tz)
    J11, J12 = fy / tz, -fy * ty / (tz * tz)
    Wm = V[:3, :3].t()
    T0 = J00[:, None] * Wm[0][None] + J02[:, None] * Wm[2][None]
    T1 = J11[:, None] * Wm[1][None] + J12[:, None] * Wm[2][None]
    S = torch.stack([cov[:, 0], cov[:, 1], cov[:, 2], cov[:, 1], cov[:, 3], cov[:, 4], cov[:, 2], cov[:, 4],
                     cov[:, 5]], 1).reshape(-1, 3, 3)
    u = (S @ T0[:, :, None])[:, :, 0]
    v = (S @ T1[:, :, None])[:, :, 0]
    a = (T0 * u).sum(1) + 0.3
    b = (T0 * v).sum(1)
    c = (T1 * v).sum(1) + 0.3
    det = a * c - b * b
    conA, conB, conC = c / det, -b / det, a / det
    with torch.no_grad():
        mid = 0.5 * (a + c)
        l1 = mid + torch.sqrt(torch.clamp(mid * mid - det, min=0.1))
        radius = torch.ceil(3.0 * torch.sqrt(l1))
        gx, gy = (W + tile - 1) // tile, (H + tile - 1) // tile
        px0, py0 = pix_x.detach(), pix_y.detach()
        x0 = torch.clamp(torch.trunc((px0 - radius) / tile), 0, gx).long()
        y0 = torch.clamp(torch.trunc((py0 - radius) / tile), 0, gy).long()
        x1 = torch.clamp(torch.trunc((px0 + radius + tile - 1) / tile), 0, gx).long()
        y1 = torch.clamp(torch.trunc((py0 + radius + tile - 1) / tile), 0, gy).long()
        visible = (tz > 0.2) & (det != 0) & ((x1 - x0) * (y1 - y0) > 0)
        radii = torch.where(visible, radius, torch.zeros_like(radius)).long()
    if colors_precomp is not None:
        rgb = colors_precomp.to(dt)
    else:
        d = p - campos.to(dt)[None]
        d = d / d.norm(dim=1, keepdim=True)
        m = (sh_degree + 1) ** 2
        B = sh_basis(sh_degree, d)
        rgb = (B[:, :, None] * shs.to(dt)[:, :m, :]).sum(1) + 0.5
        rgb = torch.clamp_min(rgb, 0.0)
    opac = opacities.to(dt).reshape(-1)
    color = torch.zeros(3, H * W, dtype=dt)
    depth_img = torch.zeros(H * W, dtype=dt)
    Tfin = torch.ones(H * W, dtype=dt)
    n_contrib = torch.zeros(H * W, dtype=torch.long)
    color_parts, depth_parts, T_parts, idx_parts = [], [], [], []
    vis_idx = torch.nonzero(visible).reshape(-1)
    order = vis_idx[torch.sort(tz.detach()[vis_idx], stable=True).indices]
    bgv = bg.to(dt)
    for ty_ in range(gy):
        for tx_ in range(gx):
            sel = order[(x0[order] <= tx_) & (x1[order] > tx_) & (y0[order] <= ty_) & (y1[order] > ty_)]
            xs = torch.arange(tx_ * tile, min((tx_ + 1) * tile, W))
            ys = torch.arange(ty_ * tile, min((ty_ + 1) * tile, H))
            yy, xx = torch.meshgrid(ys, xs, indexing="ij")
            pidx = (yy * W + xx).reshape(-1)
            if sel.numel() == 0:
                color_parts.append(bgv[:, None].expand(3, pidx.numel()))
                depth_parts.append(torch.zeros(pidx.numel(), dtype=dt))
                T_parts.append(torch.ones(pidx.numel(), dtype=dt))
                idx_parts.append(pidx)
                continue
            dx = pix_x[sel][None, :] - xx.reshape(-1, 1).to(dt)
            dy = pix_y[sel][None, :] - yy.reshape(-1, 1).to(dt)
            power = -0.5 * (conA[sel][None] * dx * dx + conC[sel][None] * dy * dy) - conB[sel][None] * dx * dy
            raw = opac[sel][None] * torch.exp(power)
            alpha = raw - (raw - 0.99).clamp(min=0).detach()
            with torch.no_grad():
                valid = (power <= 0) & (alpha >= 1.0 / 255.0)
                a_eff0 = torch.where(valid, alpha, torch.zeros_like(alpha))
                Tb = torch.cumprod(torch.cat([torch.ones_like(a_eff0[:, :1]), 1 - a_eff0[:, :-1]], 1), 1)
                stop = valid & (Tb * (1 - a_eff0) < 1e-4)
                first_stop = torch.where(stop.any(1), stop.float().argmax(1),
                                         torch.full((stop.shape[0],), stop.shape[1], dtype=torch.long))
                keep = valid & (torch.arange(stop.shape[1])[None] < first_stop[:, None])
                jidx = torch.arange(stop.shape[1])[None].expand_as(keep)
                last = torch.where(keep, jidx + 1, torch.zeros_like(jidx)).max(1).values
            a_eff = torch.where(keep, alpha, torch.zeros_like(alpha))
            one_m = 1 - a_eff
            Tb = torch.cumprod(torch.cat([torch.ones_like(one_m[:, :1]), one_m[:, :-1]], 1), 1)
            w = a_eff * Tb
            Tf = torch.prod(one_m, 1)
            col = (w[:, :, None] * rgb[sel][None]).sum(1).t() + Tf[None] * bgv[:, None]
            dep = (w * tz[sel][None]).sum(1)
            color_parts.append(col)
            depth_parts.append(dep)
            T_parts.append(Tf)
            idx_parts.append(pidx)
            n_contrib[pidx] = last
    allidx = torch.cat(idx_parts)
    inv = torch.empty_like(allidx)
    inv[allidx] = torch.arange(allidx.numel())
    color = torch.cat(color_parts, 1)[:, inv].reshape(3, H, W)
    depth_img = torch.cat(depth_parts)[inv].reshape(1, H, W)
    Tfin = torch.cat(T_parts)[inv]
    alpha_img = (1 - Tfin).reshape(1, H, W)
    return {"color": color, "depth": depth_img, "alpha": alpha_img, "radii": radii, "n_contrib": n_contrib,
            "rgb": rgb, "conic": torch.stack([conA, conB, conC], 1), "xy": torch.stack([pix_x, pix_y], 1),
            "tz": tz}
