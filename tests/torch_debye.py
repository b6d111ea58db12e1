"""Test-harness ``torch.autograd.Function`` over librsx's forward/backward pair.

Used only by the tests to check the hand-written adjoint kernel through
autograd; the library itself has no torch dependency."""
import numpy as np
import torch

from resaxs_gb300 import workloads as W


class DebyeCurve(torch.autograd.Function):
    """I(q) of body positions (N, 3) float32 through an open ``Debye`` handle."""

    @staticmethod
    def forward(ctx, xyz, handle, types):
        bodies = W.pack_bodies(xyz.detach().cpu().numpy(), types)
        iq = handle.calc(bodies)
        ctx.handle = handle
        return torch.from_numpy(iq.astype(np.float32))

    @staticmethod
    def backward(ctx, grad_iq):
        g = ctx.handle.backward(grad_iq.detach().cpu().numpy().astype(np.float32))
        return torch.from_numpy(g), None, None


def debye_curve(xyz, handle, types):
    return DebyeCurve.apply(xyz, handle, types)
