"""Autograd node shared by Scattering2D and Scattering1D.

The reference differentiates through torch autograd over its op graph, which
keeps every intermediate the backward needs (ModulusStable saves its input,
kymatio/backend/torch_backend.py:85-96).  Here the forward and backward are
single fused C-ABI calls, with two policies:

* saved form: while batch x (saved bytes per image) stays within
  ``module.activation_budget`` (4 GiB by default), the forward stores every
  order-1 and order-2 path's modulus input y (kym_*_forward_save) and the
  backward reads it (kym_*_backward_saved) with no recomputation;
* recompute form: above the budget only x is kept, and the backward
  recomputes the input and parent spectra chunk by chunk and each path's y
  (kym_*_backward).
"""
import torch

DEFAULT_ACTIVATION_BUDGET = 4 << 30


class CascadeFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, module):
        ctx.module = module
        ctx.x_shape = tuple(x.shape)
        ctx.saved_form = bool(ctx.needs_input_grad[0]) and \
            module._saved_bytes(x.shape[0]) <= module.activation_budget
        if ctx.saved_form:
            out, saved = module._forward_save_raw(x)
            ctx.save_for_backward(saved)
            return out
        ctx.save_for_backward(x)
        return module._forward_raw(x)

    @staticmethod
    def backward(ctx, grad):
        (t,) = ctx.saved_tensors
        if ctx.saved_form:
            return ctx.module._backward_saved_raw(t, grad.contiguous(), ctx.x_shape), None
        return ctx.module._backward_raw(t, grad.contiguous()), None


def forward_save(lib, prefix, module, plan, x, out_shape):
    """Runs kym_<prefix>_forward_save; returns (out, saved uint8 buffer)."""
    from . import _lib
    B = x.shape[0]
    out = torch.empty(out_shape, dtype=torch.float32, device=x.device)
    nbytes = getattr(lib, 'kym_%s_saved_bytes' % prefix)(plan.h, B)
    saved = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
    if B == 0:
        return out, saved
    with torch.cuda.device(x.device):
        ptrs = module._filter_ptrs()
        ws_bytes = getattr(lib, 'kym_%s_workspace_bytes' % prefix)(plan.h, B)
        ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=x.device)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _lib.check(getattr(lib, 'kym_%s_forward_save' % prefix)(
            plan.h, x.data_ptr(), out.data_ptr(), B, ptrs, module._n_filters, ws.data_ptr(), ws_bytes,
            saved.data_ptr(), nbytes, stream), 'kym_%s_forward_save' % prefix)
    return out, saved


def backward_saved(lib, prefix, module, plan, saved, grad, x_shape):
    """Runs kym_<prefix>_backward_saved; returns grad_x of shape x_shape."""
    from . import _lib
    B = x_shape[0]
    gx = torch.empty(x_shape, dtype=torch.float32, device=grad.device)
    if B == 0:
        return gx
    with torch.cuda.device(grad.device):
        ptrs = module._filter_ptrs()
        ws_bytes = getattr(lib, 'kym_%s_backward_workspace_bytes' % prefix)(plan.h, B)
        ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=grad.device)
        stream = torch.cuda.current_stream(grad.device).cuda_stream
        _lib.check(getattr(lib, 'kym_%s_backward_saved' % prefix)(
            plan.h, saved.data_ptr(), saved.numel(), grad.data_ptr(), gx.data_ptr(), B, ptrs, module._n_filters,
            ws.data_ptr(), ws_bytes, stream), 'kym_%s_backward_saved' % prefix)
    return gx
