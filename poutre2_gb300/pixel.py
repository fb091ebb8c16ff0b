"""Pixel processing on device images, mirroring poutre2's pixel_processing API
(include/poutre/pixel_processing/arith.hpp, compare.hpp, copy_convert.hpp) on torch CUDA tensors.

Every function runs one kernel of the C-ABI library (``pg_arith_*``, ``pg_sat_*``,
``pg_compare_image``, ``pg_copy_into``, ``pg_convert_into``) on the current CUDA stream; the
caller provides the output image.  Scalars follow the reference's ScalarTypeVariant rule in
value: they must be representable in the pixel type of the operand they stand for.
"""
from __future__ import annotations

import ctypes
import enum

import torch

from . import _lib
from .image import descriptor


class CompOpType(enum.IntEnum):
    """poutre::CompOpType (include/poutre/base/types.hpp:443-452)."""
    CompOpEqual = 1
    CompOpDiff = 2
    CompOpSup = 4
    CompOpSupEqual = 8
    CompOpInf = 16
    CompOpInfEqual = 32


def _unary(name, i_img, o_img):
    a, o = descriptor(i_img, "input"), descriptor(o_img, "output")
    _lib.call(name, ctypes.byref(a), ctypes.byref(o), _lib.current_stream())


def _binary(name, i_img1, i_img2, o_img):
    a, b, o = descriptor(i_img1, "input 1"), descriptor(i_img2, "input 2"), descriptor(o_img, "output")
    _lib.call(name, ctypes.byref(a), ctypes.byref(b), ctypes.byref(o), _lib.current_stream())


def ArithInvertImage(i_img: torch.Tensor, o_img: torch.Tensor) -> None:
    """poutre::ArithInvertImage: -v in the pixel type (src/pixel_processing/arith.cpp)."""
    _unary("pg_arith_invert_image", i_img, o_img)


def ArithSupImage(i_img1: torch.Tensor, i_img2: torch.Tensor, o_img: torch.Tensor) -> None:
    """poutre::ArithSupImage: v1 > v2 ? v1 : v2."""
    _binary("pg_arith_sup_image", i_img1, i_img2, o_img)


def ArithInfImage(i_img1: torch.Tensor, i_img2: torch.Tensor, o_img: torch.Tensor) -> None:
    """poutre::ArithInfImage: v1 < v2 ? v1 : v2."""
    _binary("pg_arith_inf_image", i_img1, i_img2, o_img)


def ArithSaturatedAddImage(i_img1: torch.Tensor, i_img2: torch.Tensor, o_img: torch.Tensor) -> None:
    """poutre::ArithSaturatedAddImage: v1 + v2 clamped to the integer type's range."""
    _binary("pg_sat_add_image", i_img1, i_img2, o_img)


def ArithSaturatedSubImage(i_img1: torch.Tensor, i_img2: torch.Tensor, o_img: torch.Tensor) -> None:
    """poutre::ArithSaturatedSubImage: v1 - v2 clamped to the integer type's range."""
    _binary("pg_sat_sub_image", i_img1, i_img2, o_img)


def ArithSaturatedAddConstant(i_img: torch.Tensor, pvalue, o_img: torch.Tensor) -> None:
    """poutre::ArithSaturatedAddConstant (src/pixel_processing/arith.cpp)."""
    a, o = descriptor(i_img, "input"), descriptor(o_img, "output")
    v = _lib.scalar(a.ptype, pvalue)
    _lib.call("pg_sat_add_constant", ctypes.byref(a), ctypes.byref(v), ctypes.byref(o), _lib.current_stream())


def ArithSaturatedSubConstant(i_img: torch.Tensor, pvalue, o_img: torch.Tensor) -> None:
    """poutre::ArithSaturatedSubConstant (src/pixel_processing/arith.cpp:471)."""
    a, o = descriptor(i_img, "input"), descriptor(o_img, "output")
    v = _lib.scalar(a.ptype, pvalue)
    _lib.call("pg_sat_sub_constant", ctypes.byref(a), ctypes.byref(v), ctypes.byref(o), _lib.current_stream())


def CompareImage(i_img: torch.Tensor, compOpType, i_comp, i_valtrue, i_valfalse, o_img: torch.Tensor) -> None:
    """poutre::CompareImage, all eight overloads (compare.hpp:31-84): o = op(i, comp) ? valtrue : valfalse.

    ``i_comp`` (the input's pixel type), ``i_valtrue`` and ``i_valfalse`` (the output's) are each a
    device image of the input's shape or a Python scalar."""
    keep = []

    a, o = descriptor(i_img, "input"), descriptor(o_img, "output")

    def operand(v, what, ptype):
        if isinstance(v, torch.Tensor):
            d = descriptor(v, what)
            keep.append(d)
            return _lib.PgOperand(ctypes.pointer(d), _lib.PgScalar())
        return _lib.PgOperand(None, _lib.scalar(ptype, v))

    c = operand(i_comp, "i_comp", a.ptype)
    t, f = operand(i_valtrue, "i_valtrue", o.ptype), operand(i_valfalse, "i_valfalse", o.ptype)
    _lib.call("pg_compare_image", ctypes.byref(a), int(CompOpType(compOpType)), ctypes.byref(c), ctypes.byref(t),
              ctypes.byref(f), ctypes.byref(o), _lib.current_stream())


def CopyInto(i_img: torch.Tensor, o_img: torch.Tensor) -> None:
    """poutre::CopyInto (src/pixel_processing/copy_convert.cpp:59): same type and shape."""
    _unary("pg_copy_into", i_img, o_img)


def ConvertInto(i_img: torch.Tensor, o_img: torch.Tensor) -> None:
    """poutre::ConvertInto (src/pixel_processing/copy_convert.cpp:301): static_cast of every pixel
    into the output's pixel type (defined for values that type holds)."""
    _unary("pg_convert_into", i_img, o_img)
