"""torch.autograd wrapper of the soft-opacity pass (vxl_trace_soft_fwd/_bwd),
kept in the test harness: the library itself exposes only the C-ABI calls.

``SoftOcclusion.apply(soft, pos, nrm, params, ctx)`` returns the image
[npix, 3]; its backward calls the hand-written adjoint kernel, which walks the
rays again instead of keeping per-ray state. ``soft`` is a contiguous float32
CUDA tensor [nz, ny, nx, 4] (opacity, albedo rgb); pos/nrm are float32
[npix, 3] G-buffer tensors and get no gradient.
"""
from __future__ import annotations

import torch

from voxelengine_gb300 import trace_soft_bwd, trace_soft_fwd


class SoftOcclusion(torch.autograd.Function):
    @staticmethod
    def forward(fctx, soft, pos, nrm, params, vctx):
        npix = pos.shape[0]
        image = torch.empty((npix, 3), device=soft.device, dtype=torch.float32)
        light = torch.empty((npix, 3), device=soft.device, dtype=torch.float32)
        trace_soft_fwd(vctx, soft, pos, nrm, npix, params, image, light)
        fctx.save_for_backward(soft, pos, nrm, light)
        fctx.params, fctx.vctx = params, vctx
        return image

    @staticmethod
    def backward(fctx, grad_image):
        soft, pos, nrm, light = fctx.saved_tensors
        grad = torch.zeros_like(soft)
        trace_soft_bwd(fctx.vctx, soft, pos, nrm, pos.shape[0], fctx.params, grad_image.contiguous(), light, grad)
        return grad, None, None, None, None


def soft_occlusion(soft, pos, nrm, params, vctx):
    return SoftOcclusion.apply(soft, pos, nrm, params, vctx)
