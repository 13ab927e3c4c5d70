"""Differentiable registration: the ECC warp residual as a torch.autograd
Function over the library's hand-written adjoint, and a joint template +
warp refinement built on it.

    r_f(x) = I_f(W(x; p_f) + u_f(x)) - T(x)      L_f = 1/2 sum_x r_f(x)^2

Forward and backward both call ``sst_warp_residual``; the backward pass
recomputes the warp from the saved inputs (no warped images are kept between
the passes). Gradients flow to the per-frame parameters, the template and
the dense flow u (e.g. a c_eccflow field).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import capi

_MODELS = {}


def _model(motion_type: int):
    if motion_type not in _MODELS:
        _MODELS[motion_type] = capi.motion(motion_type)
    return _MODELS[motion_type]


def _call(frames, template, params12, flow, motion_type, grad_loss=None, loss=None, grad_params=None,
          grad_template=None, grad_flow=None, hessian=None):
    n, h, w = frames.shape
    stream = torch.cuda.current_stream(frames.device).cuda_stream
    rc = capi.lib().sst_warp_residual(
        frames.data_ptr(), n, w, h, C.c_size_t(frames.stride(0)), template.data_ptr(), C.byref(_model(motion_type)),
        params12.data_ptr(), None if flow is None else flow.data_ptr(),
        None if grad_loss is None else grad_loss.data_ptr(), None if loss is None else loss.data_ptr(),
        None if grad_params is None else grad_params.data_ptr(),
        None if grad_template is None else grad_template.data_ptr(),
        None if grad_flow is None else grad_flow.data_ptr(), None if hessian is None else hessian.data_ptr(),
        C.c_void_p(stream))
    if rc != 0:
        raise capi.SSTError(f"sst_warp_residual: {capi.last_error()}")


def _pad12(params):
    n, M = params.shape
    p = torch.zeros((n, 12), dtype=torch.float32, device=params.device)
    p[:, :M] = params.detach().float()
    return p


class WarpResidual(torch.autograd.Function):
    """L (n,) float64 = per-frame 1/2 sum of squared residuals."""

    @staticmethod
    def forward(ctx, frames, template, params, flow, motion_type: int):
        frames = frames.detach().float().contiguous()
        template = template.detach().float().contiguous()
        fl = None if flow is None else flow.detach().float().contiguous()
        p12 = _pad12(params)
        loss = torch.empty(frames.shape[0], dtype=torch.float64, device=frames.device)
        _call(frames, template, p12, fl, motion_type, loss=loss)
        ctx.motion_type = motion_type
        ctx.M = params.shape[1]
        ctx.has_flow = flow is not None
        ctx.save_for_backward(frames, template, p12, fl if fl is not None else torch.empty(0, device=frames.device))
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        frames, template, p12, fl = ctx.saved_tensors
        fl = fl if ctx.has_flow else None
        n, h, w = frames.shape
        gl = grad_loss.detach().double().contiguous()
        gp = torch.zeros((n, 12), dtype=torch.float32, device=frames.device) if ctx.needs_input_grad[2] else None
        gt = torch.zeros((h, w), dtype=torch.float32, device=frames.device) if ctx.needs_input_grad[1] else None
        gu = (torch.zeros((n, h, w, 2), dtype=torch.float32, device=frames.device)
              if ctx.has_flow and ctx.needs_input_grad[3] else None)
        _call(frames, template, p12, fl, ctx.motion_type, grad_loss=gl, grad_params=gp, grad_template=gt,
              grad_flow=gu)
        return None, gt, None if gp is None else gp[:, :ctx.M], gu, None


def warp_residual(frames, template, params, motion_type: int, flow=None):
    """Per-frame losses with autograd to template, params and flow."""
    return WarpResidual.apply(frames, template, params, flow, motion_type)


def refine(frames, template, params, motion_type: int, flow=None, iterations: int = 5, damping: float = 1e-3):
    """Joint template + warp refinement: per iteration one Gauss-Newton step
    for every frame's parameters (J^T J and J^T r from the adjoint, LM
    damping on the diagonal) and the template's exact minimiser for fixed
    warps (the mean of the warped frames, T - dL/dT / n). Returns the refined
    (template, params) and the total loss before each step and at the end."""
    frames = frames.detach().float().contiguous()
    T = template.detach().float().clone().contiguous()
    n, h, w = frames.shape
    M = params.shape[1]
    p = params.detach().double().clone()
    fl = None if flow is None else flow.detach().float().contiguous()
    history = []
    for _ in range(iterations):
        loss = torch.empty(n, dtype=torch.float64, device=frames.device)
        g = torch.zeros((n, 12), dtype=torch.float32, device=frames.device)
        H = torch.zeros((n, 144), dtype=torch.float64, device=frames.device)
        gt = torch.zeros((h, w), dtype=torch.float32, device=frames.device)
        _call(frames, T, _pad12(p), fl, motion_type, loss=loss, grad_params=g, grad_template=gt, hessian=H)
        history.append(float(loss.sum()))
        Hm = H[:, :M * M].reshape(n, M, M)
        Hd = Hm + damping * torch.diag_embed(torch.diagonal(Hm, dim1=1, dim2=2))
        p = p - torch.linalg.solve(Hd, g[:, :M].double().unsqueeze(-1)).squeeze(-1)
        T = (T - gt / n).contiguous()
    loss = torch.empty(n, dtype=torch.float64, device=frames.device)
    _call(frames, T, _pad12(p), fl, motion_type, loss=loss)
    history.append(float(loss.sum()))
    return T, p.float(), history
