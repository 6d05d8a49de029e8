"""torch.autograd.Function over the C ABI: particle positions -> triangle
soup vertex positions, differentiable with the frame's topology held fixed
(fsr_reconstruct forward, fsr_backward backward)."""
from __future__ import annotations

import torch

from . import api


class ReconstructSurface(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz: torch.Tensor, density: torch.Tensor, rec: "api.Reconstructor", header):
        rec.reconstruct(xyz.detach(), density.detach(), header)
        pos, _ = rec.mesh_tensors()
        ctx.rec = rec
        return pos

    @staticmethod
    def backward(ctx, grad_pos: torch.Tensor):
        g = ctx.rec.backward(grad_pos)
        return g, None, None, None


def reconstruct_surface(xyz: torch.Tensor, density: torch.Tensor, rec: "api.Reconstructor", header) -> torch.Tensor:
    """Mesh vertex positions (3T, 3) of the frame; gradients flow to xyz.  The
    handle keeps the frame for the backward pass until its next frame."""
    return ReconstructSurface.apply(xyz, density, rec, header)
