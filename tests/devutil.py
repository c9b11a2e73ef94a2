"""Device-layout helpers for the GPU tests (torch is used only to hold device
memory): volume [nrays][ny] <-> [nrays][ys], sinogram [na][ny][nx] <-> [na][nx][ys]."""
import numpy as np


def vol_to_dev(plan, x):
    import torch

    t = torch.zeros(plan.nrays, plan.ys, dtype=torch.float32, device="cuda")
    t[:, :plan.ny] = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    return t


def vol_from_dev(plan, t):
    return t[:, :plan.ny].cpu().numpy()


def sino_to_dev(plan, q):
    import torch

    t = torch.zeros(plan.nangles, plan.nx, plan.ys, dtype=torch.float32, device="cuda")
    t[:, :, :plan.ny] = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda().permute(0, 2, 1)
    return t


def sino_from_dev(plan, t):
    return t[:, :, :plan.ny].permute(0, 2, 1).contiguous().cpu().numpy()


def empty_vol(plan):
    import torch

    return torch.zeros(plan.nrays, plan.ys, dtype=torch.float32, device="cuda")


def empty_sino(plan):
    import torch

    return torch.zeros(plan.nangles, plan.nx, plan.ys, dtype=torch.float32, device="cuda")
