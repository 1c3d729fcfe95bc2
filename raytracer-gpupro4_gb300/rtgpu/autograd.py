"""torch.autograd wrapper of rt_pathtrace / rt_pathtrace_adjoint, used by the
gradient harness (differentiable workload: gradients of an image loss with
respect to per-triangle albedo and the emitter radiance).

Parameterisation: emission = emitter_mask[:, None] * radiance[None, :], so
d/d radiance = the adjoint's emitter gradient.  Forward and backward both run
on the GPU through the C ABI; the backward replays the seeded paths.
"""
from __future__ import annotations

import torch

from .api import LBVH, RayTracer


class PathTraceFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo, radiance, emitter_mask, tracer: RayTracer, lbvh: LBVH, cam, spp, bounces, seed):
        emission = (emitter_mask[:, None].to(albedo.dtype) * radiance[None, :]).contiguous()
        img = tracer.pathtrace(lbvh, albedo.contiguous(), emission, cam, spp, bounces, seed)
        ctx.save_for_backward(albedo, emission)
        ctx.args = (tracer, lbvh, cam, spp, bounces, seed)
        return img

    @staticmethod
    def backward(ctx, grad_img):
        albedo, emission = ctx.saved_tensors
        tracer, lbvh, cam, spp, bounces, seed = ctx.args
        g = grad_img.contiguous().clone()
        g[:, 3] = 0.0  # alpha channel carries no gradient
        d_alb, d_le = tracer.pathtrace_adjoint(lbvh, albedo.contiguous(), emission, cam, spp, bounces, seed, g)
        return d_alb, d_le, None, None, None, None, None, None, None


def render(albedo, radiance, emitter_mask, tracer, lbvh, cam, spp, bounces, seed):
    return PathTraceFunction.apply(albedo, radiance, emitter_mask, tracer, lbvh, cam, spp, bounces, seed)
