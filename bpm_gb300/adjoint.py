"""Differentiable split-step march: d(loss)/d(dn) by the hand-written adjoint.

`propagate_exit(dn, u0, ...)` marches a batch of fields (illumination angles) through one
refractive-index volume and returns their exit planes; it is a torch.autograd.Function
whose backward is bpm_backward in libbpm_gb300.so: the forward march stores the field
every `ckpt_every` planes, the backward recomputes each segment from its checkpoint and
marches the adjoint field back with the conjugate propagator and conjugate phase masks,
writing k0 dz Im(conj(G) u) per plane. The propagator must not depend on dn, so this is
the "ignore" mean mode (the Bpm3d class semantics with prop="class", or bpm_3d's
mean_mode="ignore" with prop="functional"). The reference has no gradient
(bpm/bpm/bpm_3d_inverse.py is a non-functional sketch).
"""
import ctypes

import torch

from . import _native as N
from .bpm3d import _apply_launch, _ptr, _stream_ptr, get_plan, mask_pays, precompute_mask

__all__ = ["propagate_exit"]


class _ExitMarch(torch.autograd.Function):

    @staticmethod
    def forward(ctx, dn, u0, plan, ckpt_every, group, launch):
        B, Ny, Nx = u0.shape
        Nz = plan.size[2]
        dev = u0.device
        u0c = u0.detach().to(torch.complex64).contiguous()
        dnc = dn.detach().to(torch.float32).contiguous() if dn is not None else None
        n_ckpt = (Nz - 1) // ckpt_every + 1
        ckpt = torch.empty((B, n_ckpt, Ny, Nx), dtype=torch.complex64, device=dev)
        last = torch.empty((B, Ny, Nx), dtype=torch.complex64, device=dev)
        kind = N.DN_F32 if dnc is not None else N.DN_NONE
        bstride = Nz * Ny * Nx if (dnc is not None and dnc.dim() == 4) else 0
        # the phase masks of a shared dn, formed once for the forward march and its adjoint
        # (the same bits as forming them per element)
        mask = precompute_mask(plan, dnc, kind) if (dnc is not None and bstride == 0 and mask_pays(B, Nx, Ny)) \
            else None
        req = N.Request(B, _ptr(u0c), _ptr(dnc), kind, bstride, None, None, None, N.OUT_NONE, 0,
                        _ptr(last), None, None, 0, int(group), _ptr(ckpt), int(ckpt_every), _ptr(mask))
        _apply_launch(req, launch)
        wsb = plan.workspace_bytes(B, group)
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        N.check(N.lib().bpm_propagate(plan.handle, ctypes.byref(req), _ptr(ws), wsb, _stream_ptr()),
                "bpm_propagate")
        ctx.save_for_backward(u0c, dnc if dnc is not None else torch.empty(0, device=dev), ckpt,
                              mask if mask is not None else torch.empty(0, device=dev))
        ctx.has_mask = mask is not None
        ctx.plan = plan
        ctx.k = ckpt_every
        ctx.group = group
        ctx.launch = launch
        ctx.has_dn = dnc is not None
        ctx.bstride = bstride
        ctx.dn_dtype = dn.dtype if dn is not None else None
        return last

    @staticmethod
    def backward(ctx, grad_last):
        u0c, dnc, ckpt, mask = ctx.saved_tensors
        plan = ctx.plan
        B, Ny, Nx = u0c.shape
        Nz = plan.size[2]
        dev = u0c.device
        g = grad_last.to(torch.complex64).contiguous()
        kind = N.DN_F32 if ctx.has_dn else N.DN_NONE
        req = N.Request(B, _ptr(u0c), _ptr(dnc) if ctx.has_dn else None, kind, ctx.bstride, None, None,
                        None, N.OUT_NONE, 0, None, None, None, 0, int(ctx.group), _ptr(ckpt), int(ctx.k),
                        _ptr(mask) if ctx.has_mask else None)
        _apply_launch(req, ctx.launch)
        # a shared dn: the library sums the gradient over the fields (fixed order), so only
        # one (Nz, Ny, Nx) volume is written; plane 0 (u0, which dn does not reach) stays zero
        shared = ctx.has_dn and not ctx.bstride and 128 <= Nx <= 1024 and dnc.data_ptr() % 16 == 0
        req.grad_sum = 1 if shared else 0
        grad_dn = None
        if shared:
            grad_dn = torch.empty((Nz, Ny, Nx), dtype=torch.float32, device=dev)
            grad_dn[0].zero_()
        elif ctx.has_dn:
            grad_dn = torch.zeros((B, Nz, Ny, Nx), dtype=torch.float32, device=dev)
        grad_u0 = torch.empty((B, Ny, Nx), dtype=torch.complex64, device=dev) if ctx.needs_input_grad[1] else None
        wsb = int(N.lib().bpm_backward_workspace_bytes(plan.handle, B, int(ctx.group), int(ctx.k)))
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        N.check(N.lib().bpm_backward(plan.handle, ctypes.byref(req), _ptr(g), _ptr(grad_dn), _ptr(grad_u0),
                                     _ptr(ws), wsb, _stream_ptr()), "bpm_backward")
        gdn = None
        if ctx.has_dn and ctx.needs_input_grad[0]:
            gdn = grad_dn if (shared or ctx.bstride) else grad_dn.sum(dim=0)
            gdn = gdn.to(ctx.dn_dtype)
        return gdn, grad_u0, None, None, None, None


def propagate_exit(dn, u0, size, units, lam=.5, n0=1., absorbing_width=0, ckpt_every=16,
                   prop="functional", group=0, launch=None):
    """Exit planes (B, Ny, Nx) complex64 of the fields u0 (B, Ny, Nx) marched through dn
    (Nz, Ny, Nx) real, shared by all fields, or (B, Nz, Ny, Nx) per field. Differentiable
    in dn and u0 (torch autograd). prop = "functional" (bpm_3d, mean_mode="ignore") or
    "class" (Bpm3d's FP64 propagator). group and launch (keys conc, col_block; see
    bpm_gb300.autotune) set the launch shape of the forward and adjoint marches; they
    change no result."""
    kind = {"functional": N.PROP_FUNCTIONAL, "class": N.PROP_CLASS}[prop]
    plan = get_plan(size, units, lam, n0, absorbing_width, "ignore", kind)
    if u0.dim() == 2:
        u0 = u0.unsqueeze(0)
    Nx, Ny, Nz = plan.size
    if tuple(u0.shape[-2:]) != (Ny, Nx):
        raise ValueError("u0 must have shape (B, %d, %d)" % (Ny, Nx))
    if dn is not None and tuple(dn.shape[-3:]) != (Nz, Ny, Nx):
        raise ValueError("dn must have shape (..., %d, %d, %d)" % (Nz, Ny, Nx))
    if dn is not None and dn.is_complex():
        raise NotImplementedError("the adjoint needs real dn")
    return _ExitMarch.apply(dn, u0, plan, int(ckpt_every), int(group), dict(launch or {}))
