"""torch.autograd.Function over the C ABI: particle positions (and the particle
radius) -> triangle soup vertex positions, differentiable with the frame's
topology held fixed (fsr_reconstruct forward, fsr_backward backward).

The particle radius is the .xyz header's single radius
(FluidSurfaceReconstruction/data_format.txt:1-28), which the ZB05 and
Akinci12 fields use (updateScalarFieldValueZB05, ReconstructionCUDA.cu:
230-289); its gradient is the scalar fsr_backward returns for those fields
(0 for the anisotropic and TC01 fields, which do not use it)."""
from __future__ import annotations

from typing import Optional

import torch

from . import api


class ReconstructSurface(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz: torch.Tensor, density: torch.Tensor, radius: Optional[torch.Tensor],
                rec: "api.Reconstructor", header):
        hdr = type(header).from_buffer_copy(header)
        if radius is not None:
            hdr.particle_radius = float(radius.detach().reshape(()).item())
        rec.reconstruct(xyz.detach(), density.detach(), hdr)
        pos, _ = rec.mesh_tensors()
        ctx.rec = rec
        ctx.radius_like = radius
        return pos

    @staticmethod
    def backward(ctx, grad_pos: torch.Tensor):
        want_r = ctx.radius_like is not None and ctx.needs_input_grad[2]
        if want_r:
            g, gr = ctx.rec.backward(grad_pos, with_radius=True)
            r = ctx.radius_like
            return g, None, torch.full_like(r, gr), None, None
        return ctx.rec.backward(grad_pos), None, None, None, None


def reconstruct_surface(xyz: torch.Tensor, density: torch.Tensor, rec: "api.Reconstructor", header,
                        radius: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Mesh vertex positions (3T, 3) of the frame; gradients flow to xyz and,
    when given, to radius (a scalar tensor that replaces the header's
    particle radius).  The handle keeps the frame for the backward pass until
    its next frame."""
    return ReconstructSurface.apply(xyz, density, radius, rec, header)

