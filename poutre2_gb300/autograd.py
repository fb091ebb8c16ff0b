"""Differentiable flat morphology on float32 tensors (torch.autograd.Function).

Flat dilation / erosion by a (2r+1) x (2r+1) square over the last two dimensions of an
[..., H, W] float32 CUDA tensor, and opening / closing built from them.  The adjoint routes
each upstream gradient to the first-in-scan-order (dy-major, then dx) arg-extremum of the
clipped window; it recomputes that arg in backward instead of storing it and accumulates by
a gather (deterministic, no atomics).  No counterpart in the reference; the forward equals
poutre::Dilate/Erode by the square (SESquare2D iterated r times).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


def _stream():
    return _lib.current_stream()


def _planes(x: torch.Tensor):
    if x.dtype != torch.float32 or not x.is_cuda or x.ndim < 2:
        raise _lib.PoutreError(1, "flat morphology autograd expects a float32 CUDA tensor [..., H, W]")
    H, W = x.shape[-2], x.shape[-1]
    return x.numel() // max(H * W, 1), H, W


def flat_forward(x: torch.Tensor, r: int, dilate: bool) -> torch.Tensor:
    x = x.contiguous()
    y = torch.empty_like(x)
    P, H, W = _planes(x)
    _lib.call("pg_flat_morph2d_forward", x.data_ptr(), y.data_ptr(), P, H, W, r, r, int(dilate), _stream())
    return y


def flat_backward(x: torch.Tensor, gy: torch.Tensor, r: int, dilate: bool) -> torch.Tensor:
    x = x.contiguous()
    gy = gy.contiguous()
    gx = torch.empty_like(x)
    P, H, W = _planes(x)
    _lib.call("pg_flat_morph2d_backward", x.data_ptr(), gy.data_ptr(), gx.data_ptr(), P, H, W, r, r, int(dilate),
              _stream())
    return gx


def flat_forward_arg(x: torch.Tensor, r: int, dilate: bool):
    """Forward that also returns the arg codes (uint8, one per pixel) the backward gathers from."""
    x = x.contiguous()
    y = torch.empty_like(x)
    code = torch.empty(x.shape, dtype=torch.uint8, device=x.device)
    P, H, W = _planes(x)
    _lib.call("pg_flat_morph2d_forward_arg", x.data_ptr(), y.data_ptr(), code.data_ptr(), P, H, W, r, int(dilate),
              _stream())
    return y, code


def flat_backward_arg(code: torch.Tensor, gy: torch.Tensor, r: int) -> torch.Tensor:
    gy = gy.contiguous()
    gx = torch.empty_like(gy)
    P, H, W = _planes(gy)
    _lib.call("pg_flat_morph2d_backward_arg", code.data_ptr(), gy.data_ptr(), gx.data_ptr(), P, H, W, r, _stream())
    return gx


def _saves_arg(r: int) -> bool:
    return 1 <= r <= 3  # the saved-arg kernels' window sizes; others recompute the arg in backward


class FlatMorph(torch.autograd.Function):
    """y = dilate_r(x) or erode_r(x).  With a gradient wanted, the forward saves the arg codes (one
    byte per pixel) and the backward gathers from them; otherwise x is kept and the arg recomputed."""

    @staticmethod
    def forward(ctx, x, r: int, dilate: bool):
        ctx.r, ctx.dilate = int(r), bool(dilate)
        ctx.arg = ctx.needs_input_grad[0] and _saves_arg(ctx.r)
        if ctx.arg:
            y, code = flat_forward_arg(x, ctx.r, ctx.dilate)
            ctx.save_for_backward(code)
            return y
        ctx.save_for_backward(x)
        return flat_forward(x, ctx.r, ctx.dilate)

    @staticmethod
    def backward(ctx, gy):
        (saved,) = ctx.saved_tensors
        if ctx.arg:
            return flat_backward_arg(saved, gy, ctx.r), None, None
        return flat_backward(saved, gy, ctx.r, ctx.dilate), None, None


class FlatOpenClose(torch.autograd.Function):
    """Opening (dilate o erode) or closing (erode o dilate).  With a gradient wanted, both passes save
    their arg codes; otherwise the intermediate image is kept and the arg indices are recomputed."""

    @staticmethod
    def forward(ctx, x, r: int, opening: bool):
        first_dilate = not opening
        ctx.r, ctx.first_dilate = int(r), first_dilate
        ctx.arg = ctx.needs_input_grad[0] and _saves_arg(ctx.r)
        if ctx.arg:
            mid, c1 = flat_forward_arg(x, ctx.r, first_dilate)
            y, c2 = flat_forward_arg(mid, ctx.r, not first_dilate)
            ctx.save_for_backward(c1, c2)
            return y
        mid = flat_forward(x, r, first_dilate)
        y = flat_forward(mid, r, not first_dilate)
        ctx.save_for_backward(x, mid)
        return y

    @staticmethod
    def backward(ctx, gy):
        if ctx.arg:
            c1, c2 = ctx.saved_tensors
            return flat_backward_arg(c1, flat_backward_arg(c2, gy, ctx.r), ctx.r), None, None
        x, mid = ctx.saved_tensors
        g_mid = flat_backward(mid, gy, ctx.r, not ctx.first_dilate)
        return flat_backward(x, g_mid, ctx.r, ctx.first_dilate), None, None


def dilation(x, r: int = 2):
    return FlatMorph.apply(x, r, True)


def erosion(x, r: int = 2):
    return FlatMorph.apply(x, r, False)


def opening(x, r: int = 2):
    return FlatOpenClose.apply(x, r, True)


def closing(x, r: int = 2):
    return FlatOpenClose.apply(x, r, False)
