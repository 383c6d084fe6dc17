"""Thin torch binding of the forward marcher and the backward kernel.

``RenderFunction.apply(renderer, views, colours, xyz, radii)`` renders the
views with the renderer's current cloud and returns (rgb [P, 3], depth [P],
hit [P]) for all pixels of all views concatenated (row 0 of each view is
its bottom row).  Backward calls ``rm_backward``: gradients w.r.t. float32
colours, positions and radii through each pixel's stored hit index (see
include/rm.h).  ``colours``/``xyz``/``radii`` are the leaf tensors the
gradients are reported for; they must describe the cloud the renderer
holds (the forward does not re-upload them).
"""
from __future__ import annotations

import torch


class RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, renderer, views, colours, xyz, radii):
        dev = colours.device
        rgb_parts, depth_parts, hit_parts = [], [], []
        for v in views:
            frame = {"rgbd": torch.empty((v.height, v.width, 4), dtype=torch.float32, device=dev),
                     "hit": torch.empty((v.height, v.width), dtype=torch.int32, device=dev)}
            renderer.render_into(v, frame, device=True)
            rgb_parts.append(frame["rgbd"].reshape(-1, 4)[:, :3])
            depth_parts.append(frame["rgbd"].reshape(-1, 4)[:, 3])
            hit_parts.append(frame["hit"].reshape(-1))
        renderer.synchronize()
        rgb = torch.cat(rgb_parts).contiguous()
        depth = torch.cat(depth_parts).contiguous()
        hit = torch.cat(hit_parts).contiguous()
        ctx.renderer = renderer
        ctx.views = views
        ctx.n = xyz.shape[0]
        ctx.save_for_backward(hit)
        ctx.mark_non_differentiable(hit)
        return rgb, depth, hit

    @staticmethod
    def backward(ctx, g_rgb, g_depth, g_hit):
        (hit,) = ctx.saved_tensors
        dev = hit.device
        if g_rgb is None:
            g_rgb = torch.zeros((hit.shape[0], 3), dtype=torch.float32, device=dev)
        if g_depth is None:
            g_depth = torch.zeros(hit.shape[0], dtype=torch.float32, device=dev)
        g_rgb = g_rgb.to(torch.float32).contiguous()
        g_depth = g_depth.to(torch.float32).contiguous()
        n = ctx.n
        gc = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        gx = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        gr = torch.zeros(n, dtype=torch.float32, device=dev)
        torch.cuda.current_stream(dev).synchronize()
        ctx.renderer.backward(ctx.views, g_rgb, g_depth, hit, gc, gx, gr)
        ctx.renderer.synchronize()
        return None, None, gc, gx, gr


def render(renderer, views, colours, xyz, radii):
    return RenderFunction.apply(renderer, views, colours, xyz, radii)
