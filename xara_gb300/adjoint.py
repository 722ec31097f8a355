"""Gradients of a transient response with respect to material parameters,
as a ``torch.autograd.Function``.

The forward pass runs a Newmark analysis of a force-based frame model on
the GPU from its initial state (the device Newton driver, checkpointing the
committed state every ``ckpt_every`` steps) and returns

    J = sum over steps n and terms k of weight_k * u(node_k, dof_k, t_n)^2;

the backward pass is the library's reverse sweep (``xg_adjoint_backward``),
which recomputes each segment from its checkpoint and sweeps it backwards
through the Newmark step, the force-based elements' compatibility state and
the fibers' laws.  Forward-mode AD (``torch.func.jvp``, dual tensors of
``torch.autograd.forward_ad``) runs the library's direct differentiation
(``xg_ddm_forward``) along the tangent of ``theta`` from the initial state
instead.  ``theta`` holds the first three parameters of every uniaxial
material ([num_uni, 3]; Steel02: Fy, E0, b), float64 on any device.  PyTorch
only carries the parameters, the tangents and the gradient; all work runs in
``libxara_gpu.so``.
"""
import numpy as np
import torch

from . import gpu
from ._abi import XG_UNI_NPARAM


class FrameResponse(torch.autograd.Function):
    """J(theta) for a :class:`xara_gb300.gpu.DeviceModel` of frames."""

    @staticmethod
    def forward(ctx, theta, model, phase, num_steps, ckpt_every, objective):
        q = np.array(model.desc.uni_param, np.float64).reshape(-1, XG_UNI_NPARAM)
        t = theta.detach().to("cpu", torch.float64).numpy()
        if t.shape != (q.shape[0], 3):
            raise ValueError(f"theta must be [{q.shape[0]}, 3]")
        q[:, :3] = t
        gpu.set_uniaxial_params(model, q)
        node, dof, weight = objective
        J = gpu.adjoint_forward(model, phase, num_steps, ckpt_every, node, dof, weight)
        ctx.model = model
        ctx.phase, ctx.num_steps, ctx.objective = phase, num_steps, objective
        ctx.theta_device, ctx.theta_dtype = theta.device, theta.dtype
        return torch.tensor(J, dtype=torch.float64, device=theta.device)

    @staticmethod
    def jvp(ctx, dtheta, *_):
        """dJ along dtheta: the DDM of the same run from the initial state."""
        t = dtheta.detach().to("cpu", torch.float64).numpy().reshape(1, -1, 3)
        ctx.model.reset()
        node, dof, weight = ctx.objective
        _, dJ = gpu.ddm_forward(ctx.model, ctx.phase, ctx.num_steps, t, node, dof, weight)
        return torch.tensor(dJ[0], dtype=torch.float64, device=ctx.theta_device)

    @staticmethod
    def backward(ctx, grad_J):
        g = gpu.adjoint_backward(ctx.model, float(grad_J))
        grad = torch.from_numpy(g).to(ctx.theta_device, ctx.theta_dtype)
        return grad, None, None, None, None, None


def frame_response(theta, model, phase, num_steps, ckpt_every, objective):
    """J(theta); differentiable in theta (see :class:`FrameResponse`)."""
    return FrameResponse.apply(theta, model, phase, num_steps, ckpt_every, objective)
