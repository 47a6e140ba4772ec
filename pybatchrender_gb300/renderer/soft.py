"""Differentiable soft-coverage rendering as a ``torch.autograd.Function``.

The forward launches the soft raster kernel (float32 ``[N,3,H,W]`` plus
per-pixel log-sum-exp statistics); the backward launches the hand-written
adjoint kernel, which recomputes the fragment lists and returns gradients for
every geometry node's ``pos``, ``hpr``, ``scale`` and ``color`` tensors and for
the light direction.  The soft model is described in ``include/pbr_capi.h``
(``pbr_soft_config``); it has no counterpart in the reference.
"""
from __future__ import annotations

import torch

from .. import _capi


class SoftRasterize(torch.autograd.Function):
    @staticmethod
    def forward(ctx, renderer, light_dir: torch.Tensor, *params: torch.Tensor) -> torch.Tensor:
        out, stats = renderer._soft_forward(light_dir)
        ctx.renderer = renderer
        ctx.save_for_backward(out, stats, light_dir)
        return out

    @staticmethod
    def backward(ctx, gout: torch.Tensor):
        out, stats, light_dir = ctx.saved_tensors
        r = ctx.renderer
        node_grads, g_hat = r._soft_backward(out, stats, gout.contiguous())
        L = light_dir.detach().to(g_hat.device, torch.float32)
        n = torch.linalg.norm(L)
        Ln = L / n
        g_light = (g_hat - torch.dot(g_hat, Ln) * Ln) / n
        flat = []
        for g in node_grads:
            flat.extend(g)
        return (None, g_light.to(light_dir.device, light_dir.dtype), *flat)


def soft_params(renderer) -> list[torch.Tensor]:
    """The tensors the soft render is differentiable in, node by node:
    ``pos [B,3], hpr [B,3], scale [B], color [B,4]``."""
    out = []
    for node in renderer._node_ids:
        out += [node.pos, node.hpr, node.scale, node.color]
    return out


def soft_render(renderer, light_dir: torch.Tensor | None = None) -> torch.Tensor:
    """Differentiable soft render of ``renderer``'s current scene.  Gradients
    flow to any node tensor with ``requires_grad`` and to ``light_dir`` (a
    3-vector; defaults to the light's current direction)."""
    if light_dir is None:
        light = renderer._pbr_light
        d = light.dir_dir if light is not None else (0.0, 0.0, 1.0)
        light_dir = torch.tensor(d, dtype=torch.float32)
    return SoftRasterize.apply(renderer, light_dir, *soft_params(renderer))


def call(renderer, name: str, *args) -> None:
    _capi.call(renderer._lib, renderer._ctx, name, *args)
