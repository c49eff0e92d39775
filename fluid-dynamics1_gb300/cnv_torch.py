"""torch.autograd.Function over libcnv's adjoint (cnv_adjoint_*), through the ctypes binding.

    w_final = CavityRollout.apply(w0, lid, adjoint, nsteps)

maps the initial vorticity w0 (n x n float64 CUDA tensor) and the lid speed (0-d float64
tensor) to the vorticity after nsteps time steps. Its backward calls the hand-written adjoint
kernels (cnv_adjoint_backward_device), which recompute the forward steps from the checkpoints
the forward call kept. It exists to check the library's gradients against finite differences
and to let a PyTorch objective drive them; all the arithmetic happens in libcnv.so.
"""
from __future__ import annotations

import torch

import cnvpy


class CavityRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w0: torch.Tensor, lid: torch.Tensor, adjoint: cnvpy.Adjoint, nsteps: int):
        if not w0.is_cuda or w0.dtype != torch.float64 or w0.dim() != 2:
            raise TypeError("w0 must be a 2-D float64 CUDA tensor")
        w0c = w0.detach().contiguous()
        lid_v = float(lid.detach().cpu())
        w_final = torch.empty_like(w0c)
        torch.cuda.synchronize(w0c.device)  # the library runs on its own stream
        adjoint.forward_device(w0c.data_ptr(), lid_v, nsteps, w_final.data_ptr())
        ctx.adjoint, ctx.nsteps, ctx.lid, ctx.generation = adjoint, nsteps, lid_v, adjoint.generation
        ctx.save_for_backward(w0c)
        return w_final

    @staticmethod
    def backward(ctx, g_final: torch.Tensor):
        (w0c,) = ctx.saved_tensors
        adj = ctx.adjoint
        g = g_final.detach().contiguous().to(torch.float64)
        torch.cuda.synchronize(g.device)
        if adj.generation != ctx.generation:
            # another forward run replaced the checkpoints: run this one again
            scratch = torch.empty_like(w0c)
            adj.forward_device(w0c.data_ptr(), ctx.lid, ctx.nsteps, scratch.data_ptr())
        g_w0 = torch.empty_like(w0c)
        g_lid = adj.backward_device(g.data_ptr(), g_w0.data_ptr())
        return g_w0, torch.tensor(g_lid, dtype=torch.float64, device=w0c.device), None, None


def enstrophy(w: torch.Tensor, h2: float) -> torch.Tensor:
    """J = 1/2 sum w^2 dx dy."""
    return 0.5 * h2 * (w * w).sum()
