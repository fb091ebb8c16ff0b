"""low_level_morpho on device images, mirroring poutre2's public API.

Names, argument order and meaning follow include/poutre/low_level_morpho/ero_dil.hpp:32-47
and ero_dil_line.hpp:32-47: the caller provides the output image, which must have the
input's shape and type and be a distinct buffer; errors raise ``PoutreError`` where the
reference throws.  Opening / closing / gradient are additions (the reference announces them
in low_level_morpho.hpp:15 but has none).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .image import descriptor
from .se import Common_NL_SE, Compound_NL_SE, NeighborList


def _stream():
    return _lib.current_stream()


def _offsets(nl: NeighborList, rank: int):
    if nl.rank != rank:
        raise _lib.PoutreError(3, "Dilate Unsupported IStructuringElement type (SE rank differs from image rank)")
    flat = [v for o in nl.offsets for v in o]
    arr = (ctypes.c_int32 * len(flat))(*flat)
    return arr, len(nl.offsets)


def _erode_dilate(i_img, se, param, o_img, dilate: bool):
    di, do = descriptor(i_img, "input"), descriptor(o_img, "output")
    if isinstance(se, Compound_NL_SE):
        _lib.call("pg_dilate_compound" if dilate else "pg_erode_compound", ctypes.byref(di), int(se), int(param),
                  ctypes.byref(do), _stream())
    elif isinstance(se, NeighborList):
        arr, n = _offsets(se, i_img.ndim)
        _lib.call("pg_dilate_nl" if dilate else "pg_erode_nl", ctypes.byref(di), arr, n, ctypes.byref(do), _stream())
    else:
        _lib.call("pg_dilate" if dilate else "pg_erode", ctypes.byref(di), int(Common_NL_SE(se)), int(param),
                  ctypes.byref(do), _stream())


def Erode(i_img: torch.Tensor, se, iter_or_img=None, o_img: torch.Tensor | None = None):
    """poutre::Erode overloads:
    ``Erode(i_img, Common_NL_SE, iter, o_img)``, ``Erode(i_img, Compound_NL_SE, size, o_img)``,
    ``Erode(i_img, NeighborList, o_img)``."""
    if isinstance(se, NeighborList):
        _erode_dilate(i_img, se, 0, iter_or_img, False)
    else:
        _erode_dilate(i_img, se, iter_or_img, o_img, False)


def Dilate(i_img: torch.Tensor, se, iter_or_img=None, o_img: torch.Tensor | None = None):
    """poutre::Dilate overloads (see Erode)."""
    if isinstance(se, NeighborList):
        _erode_dilate(i_img, se, 0, iter_or_img, True)
    else:
        _erode_dilate(i_img, se, iter_or_img, o_img, True)


def _line(name, i_img, half, o_img):
    di, do = descriptor(i_img, "input"), descriptor(o_img, "output")
    _lib.call(name, ctypes.byref(di), int(half), ctypes.byref(do), _stream())


def ErodeX(i_img, size_half_segment: int, o_img):
    _line("pg_erode_x", i_img, size_half_segment, o_img)


def DilateX(i_img, size_half_segment: int, o_img):
    _line("pg_dilate_x", i_img, size_half_segment, o_img)


def ErodeY(i_img, size_half_segment: int, o_img):
    _line("pg_erode_y", i_img, size_half_segment, o_img)


def DilateY(i_img, size_half_segment: int, o_img):
    _line("pg_dilate_y", i_img, size_half_segment, o_img)


# ----------------------------------------------------------------------------- SE descriptors
def se_static(common_se, iterations: int = 1) -> _lib.PgSE:
    s = _lib.PgSE()
    s.kind, s.common_se, s.iter = 0, int(common_se), int(iterations)
    return s


def se_rect(hy: int, hx: int) -> _lib.PgSE:
    """(2hy+1) x (2hx+1) flat rectangle (31x31 square: se_rect(15, 15))."""
    s = _lib.PgSE()
    s.kind, s.hy, s.hx = 1, int(hy), int(hx)
    return s


def se_line(dy: int, dx: int, half: int) -> _lib.PgSE:
    """Segment t*(dy,dx), t in [-half, half]: (0,1) horizontal, (1,0) vertical, (-1,1) 45 degrees."""
    s = _lib.PgSE()
    s.kind, s.dy, s.dx, s.half = 2, int(dy), int(dx), int(half)
    return s


def se_nl(nl: NeighborList):
    flat = [v for o in nl.offsets for v in o]
    arr = (ctypes.c_int32 * len(flat))(*flat)
    s = _lib.PgSE()
    s.kind, s.offsets, s.n = 3, arr, len(nl.offsets)
    s._keep = arr  # keep the host array alive with the descriptor
    return s


def _as_se(se) -> _lib.PgSE:
    if isinstance(se, _lib.PgSE):
        return se
    if isinstance(se, NeighborList):
        return se_nl(se)
    return se_static(se, 1)


def _composite(name, i_img, se, o_img):
    di, do = descriptor(i_img, "input"), descriptor(o_img, "output")
    s = _as_se(se)
    _lib.call(name, ctypes.byref(di), ctypes.byref(s), ctypes.byref(do), _stream())


def ErodeSE(i_img, se, o_img):
    _composite("pg_erode_se", i_img, se, o_img)


def DilateSE(i_img, se, o_img):
    _composite("pg_dilate_se", i_img, se, o_img)


def Opening(i_img, se, o_img):
    """dilate(erode(i_img)) by the same SE."""
    _composite("pg_opening", i_img, se, o_img)


def Closing(i_img, se, o_img):
    """erode(dilate(i_img)) by the same SE."""
    _composite("pg_closing", i_img, se, o_img)


def Gradient(i_img, se, o_img):
    """dilate(i_img) - erode(i_img) (plain difference)."""
    _composite("pg_gradient", i_img, se, o_img)
