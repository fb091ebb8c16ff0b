"""Connected-component labelling on device images, mirroring poutre2's label module.

``label_binary`` / ``label_flat_zones`` follow include/poutre/label/label_binary.hpp and
label_flat_zones.hpp: the caller provides an int64 output image of the input's shape; components
are numbered 1.. by the raster position of their first pixel (0 = background) and the number of
labels is returned, as the reference's ``size_t``.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .image import descriptor
from .se import Common_NL_SE


def _label(name, i_img: torch.Tensor, nl_static, o_img: torch.Tensor) -> int:
    di, do = descriptor(i_img, "input"), descriptor(o_img, "output")
    n = ctypes.c_int64(0)
    _lib.call(name, ctypes.byref(di), int(Common_NL_SE(nl_static)), ctypes.byref(do), ctypes.byref(n),
              _lib.current_stream())
    return int(n.value)


def label_binary(i_img: torch.Tensor, nl_static, o_img: torch.Tensor) -> int:
    """poutre::label::label_binary(i_img, Common_NL_SE, o_img) -> number of labels
    (src/label/label_binary.cpp): foreground = pixels != 0 joined to earlier neighbours > 0."""
    return _label("pg_label_binary", i_img, nl_static, o_img)


def label_flat_zones(i_img: torch.Tensor, nl_static, o_img: torch.Tensor) -> int:
    """poutre::label::label_flat_zones(i_img, Common_NL_SE, o_img) -> number of labels
    (src/label/label_flat_zones.cpp): every pixel, joined to equal neighbours."""
    return _label("pg_label_flat_zones", i_img, nl_static, o_img)


def label_minima(i_img: torch.Tensor, nl_static, o_img: torch.Tensor) -> int:
    """poutre::label::label_minima(i_img, Common_NL_SE, o_img) (src/label/label_extrema.cpp):
    label_binary of h_concave(i_img, 1); returns the number of labels (the reference returns none)."""
    return _label("pg_label_minima", i_img, nl_static, o_img)


def label_maxima(i_img: torch.Tensor, nl_static, o_img: torch.Tensor) -> int:
    """poutre::label::label_maxima(i_img, Common_NL_SE, o_img): label_binary of h_convex(i_img, 1)."""
    return _label("pg_label_maxima", i_img, nl_static, o_img)
