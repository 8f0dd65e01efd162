"""Differentiable dirty imaging: ``torch.autograd.Function`` over the plan.

Forward: image = A(V), the w-stacking imaging operator (grid -> per-plane FFT
-> w-correction) applied to the folded measurement values
V_m = sum_{f,p} weight[m,p] * vis[m,f,p] (NaN-flagged entries skipped, as in
w-stacking.cu:98-112).  The image is returned as a real tensor [ny, nx, 2].

Backward: the hand-written adjoint A^H (w-correction adjoint -> per-plane FFT
with exponent -i -> degridding), reusing the binning of the forward.  With
g = A^H(dL/dI) (complex per measurement):
    dL/dvis_real[m,f,p] = weight[m,p] * Re g_m
    dL/dvis_img[m,f,p]  = weight[m,p] * Im g_m
    dL/dweight[m,p]     = sum_f (Re g_m * vis_real[m,f,p] + Im g_m * vis_img[m,f,p])
for entries whose vis_real is not NaN, zero otherwise.  Image pixels where the
reference's w-correction is undefined (sin^2 + sin^2 > 1, NaN in the forward
image) are excluded from the adjoint.
"""
from __future__ import annotations

import torch

from .api import Plan


class WStackImage(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vis_real, vis_img, weight, plan: Plan, uu, vv, ww, freq_per_chan: int = 1,
                polarizations: int = 1):
        image = plan.image_forward(uu, vv, ww, vis_real.detach(), vis_img.detach(),
                                   weight.detach(), freq_per_chan, polarizations)
        ctx.plan = plan
        ctx.geom = (uu, vv, ww)
        ctx.fp = (int(freq_per_chan), int(polarizations))
        ctx.token = id(plan._keep)
        ctx.save_for_backward(vis_real, vis_img, weight)
        return torch.view_as_real(image)

    @staticmethod
    def backward(ctx, grad_image):
        plan: Plan = ctx.plan
        vr, vi, wt = ctx.saved_tensors
        nf, np_ = ctx.fp
        if id(plan._keep) != ctx.token:
            # the plan binned another batch since this forward: bin again
            uu, vv, ww = ctx.geom
            plan.bin(uu, vv, ww, vr.detach(), vi.detach(), wt.detach(), nf, np_)
            ctx.token = id(plan._keep)
        r = torch.view_as_complex(grad_image.to(torch.float64 if plan.cdtype == torch.complex128
                                                else torch.float32).contiguous())
        g = plan.image_adjoint(r)
        n = g.shape[0]
        gr = g.real.reshape(n, 1, 1)
        gi = g.imag.reshape(n, 1, 1)
        vr3 = vr.detach().reshape(n, nf, np_)
        vi3 = vi.detach().reshape(n, nf, np_)
        wt3 = wt.detach().reshape(n, 1, np_)
        ok = ~torch.isnan(vr3)
        d_vr = d_vi = d_wt = None
        if ctx.needs_input_grad[0]:
            d_vr = torch.where(ok, wt3 * gr, 0).to(vr.dtype).reshape(vr.shape)
        if ctx.needs_input_grad[1]:
            d_vi = torch.where(ok, wt3 * gi, 0).to(vi.dtype).reshape(vi.shape)
        if ctx.needs_input_grad[2]:
            t = torch.where(ok, gr * vr3 + gi * vi3, 0).sum(dim=1)
            d_wt = t.to(wt.dtype).reshape(wt.shape)
        return d_vr, d_vi, d_wt, None, None, None, None, None, None


def dirty_image(plan: Plan, uu, vv, ww, vis_real, vis_img, weight, freq_per_chan=1,
                polarizations=1):
    """Differentiable dirty image [ny, nx, 2] (real, imag) of the measurements."""
    return WStackImage.apply(vis_real, vis_img, weight, plan, uu, vv, ww, freq_per_chan,
                             polarizations)
