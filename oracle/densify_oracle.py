"""Test infrastructure only (the oracle): the reference's densify_and_prune
(scene/gaussian_model_cf.py:628-694, with densification_postfix :605-626, prune_points
:560-575, cat_tensors_to_optimizer :576-603 and build_rotation of
utils/general_utils.py:76-97) restated in PyTorch on the CPU, float32 as the reference
computes, with the split samples taken as std * z from given standard-normal draws z
(the reference's torch.normal(mean=0, std) is std * z of its own draws). Runs on the
device of its inputs (the benchmark times it on the GPU as the PyTorch formulation)."""
from __future__ import annotations

import torch

GROUPS = ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation")


def build_rotation(r: torch.Tensor) -> torch.Tensor:
    norm = torch.sqrt(r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1] + r[:, 2] * r[:, 2] + r[:, 3] * r[:, 3])
    q = r / norm[:, None]
    R = torch.zeros((q.size(0), 3, 3), dtype=r.dtype, device=r.device)
    r_, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - r_ * z)
    R[:, 0, 2] = 2 * (x * z + r_ * y)
    R[:, 1, 0] = 2 * (x * y + r_ * z)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - r_ * x)
    R[:, 2, 0] = 2 * (x * z - r_ * y)
    R[:, 2, 1] = 2 * (y * z + r_ * x)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def densify_and_prune(params: dict, exp_avg: dict, exp_avg_sq: dict, grad_accum, denom, max_grad, min_opacity,
                      extent, max_screen_size, percent_dense, z):
    """Returns (params, exp_avg, exp_avg_sq) after densify_and_prune; z [2, splits, 3]."""
    P = {k: v.clone() for k, v in params.items()}
    M = {k: v.clone() for k, v in exp_avg.items()}
    V = {k: v.clone() for k, v in exp_avg_sq.items()}
    grads = (grad_accum / denom)[:, None]
    grads[grads.isnan()] = 0.0

    def cat(d):
        for k in GROUPS:
            M[k] = torch.cat((M[k], torch.zeros_like(d[k])))
            V[k] = torch.cat((V[k], torch.zeros_like(d[k])))
            P[k] = torch.cat((P[k], d[k]))

    def prune(mask):
        keep = ~mask
        for k in GROUPS:
            P[k], M[k], V[k] = P[k][keep], M[k][keep], V[k][keep]

    scale = lambda: torch.exp(P["scaling"])  # noqa: E731
    # densify_and_clone
    sel = torch.norm(grads, dim=-1) >= max_grad
    sel = sel & (torch.max(scale(), dim=1).values <= percent_dense * extent)
    cat({k: P[k][sel] for k in GROUPS})
    # densify_and_split (N = 2)
    n_init = P["xyz"].shape[0]
    padded = torch.zeros(n_init, device=grads.device)
    padded[:grads.shape[0]] = grads.squeeze()
    sel = (padded >= max_grad) & (torch.max(scale(), dim=1).values > percent_dense * extent)
    stds = scale()[sel].repeat(2, 1)
    samples = stds * z.reshape(-1, 3)
    rots = build_rotation(P["rotation"][sel]).repeat(2, 1, 1)
    new = {"xyz": torch.bmm(rots, samples.unsqueeze(-1)).squeeze(-1) + P["xyz"][sel].repeat(2, 1),
           "scaling": torch.log(scale()[sel].repeat(2, 1) / (0.8 * 2)),
           "rotation": P["rotation"][sel].repeat(2, 1), "f_dc": P["f_dc"][sel].repeat(2, 1, 1),
           "f_rest": P["f_rest"][sel].repeat(2, 1, 1), "opacity": P["opacity"][sel].repeat(2, 1)}
    cat(new)
    prune(torch.cat((sel, torch.zeros(2 * int(sel.sum()), dtype=torch.bool, device=sel.device))))
    # prune (max_radii2D is zero after densification_postfix)
    mask = (torch.sigmoid(P["opacity"]) < min_opacity).squeeze()
    if max_screen_size:
        mask = mask | (torch.max(scale(), dim=1).values > 0.1 * extent)
    prune(mask)
    return P, M, V
