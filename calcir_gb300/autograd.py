"""torch.autograd wrapper of the C-ABI backward entry (cir_loss_grad), used to check the
adjoint gradient: SpectrumLoss.apply(theta, engine, xyz, box, frame_of_step, target_ir,
target_vv) returns the spectrum-mismatch loss as a 0-d float64 tensor whose backward gives
dL/dtheta from the library's adjoint (no autograd graph is built through the CUDA path)."""
from __future__ import annotations

import numpy as np
import torch


class SpectrumLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, engine, xyz, box, frame_of_step, target_ir, target_vv):
        engine.set_coeffs(theta.detach().cpu().numpy().astype(np.float32))
        loss, grad = engine.loss_grad(xyz, box, frame_of_step, target_ir, target_vv)
        ctx.save_for_backward(torch.as_tensor(grad, dtype=theta.dtype, device=theta.device))
        return torch.as_tensor(loss, dtype=torch.float64, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        (grad,) = ctx.saved_tensors
        return grad_out * grad, None, None, None, None, None, None
