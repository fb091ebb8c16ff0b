"""pypoutre's Python names over the GB300 library: a drop-in for poutre2's nanobind module
(python/main.cpp:27) on device images.

The function names, argument order and enums follow python/base, python/pixel_processing,
python/structuring_element, python/low_level_morpho, python/geodesy and python/label.  Images are
``Image`` objects wrapping a contiguous CUDA tensor; every function also takes a torch CUDA tensor,
or any object that exports a CUDA buffer through DLPack, without copying it.  Outputs are written
in place and functions return None, as in pypoutre; factories return new ``Image`` objects.

Differences from pypoutre, each on purpose:
  * ``h_maxima`` is bound under its own name (pypoutre registers it as a second "h_minima",
    python/geodesy/geodesy.cpp:19-20, so pypoutre's h_maxima is unreachable);
  * ``reconstruction`` is exported (pypoutre binds no geodesic reconstruction);
  * the RecType values stay inside ``RecType`` (pypoutre's ``export_values`` puts ``dilate`` /
    ``erode`` at module level, where the morphology functions of the same names live);
  * ``PType.GrayUINT16`` exists (the reference has no 16-bit pixel type);
  * io (OIIO / HDF5 loaders) is not provided; ``from_numpy`` / ``Image.numpy`` move host arrays.
"""
from __future__ import annotations

import enum

import numpy as np
import torch

from . import geo as _geo
from . import image as _image
from . import label as _label
from . import llm as _llm
from . import pixel as _pixel
from .se import Common_NL_SE, Compound_NL_SE


# ----------------------------------------------------------------------------- enums (python/base/types.cpp)
class PType(enum.IntEnum):
    GrayUINT8 = int(_image.PType.PType_GrayUINT8)
    GrayINT32 = int(_image.PType.PType_GrayINT32)
    GrayINT64 = int(_image.PType.PType_GrayINT64)
    F32 = int(_image.PType.PType_F32)
    D64 = int(_image.PType.PType_D64)
    GrayUINT16 = int(_image.PType.PType_GrayUINT16)


class CType(enum.IntEnum):
    """poutre::CompoundType; only Scalar images exist on the device."""
    Scalar = 1


class Comp(enum.IntEnum):
    Diff = int(_pixel.CompOpType.CompOpDiff)
    Equal = int(_pixel.CompOpType.CompOpEqual)
    Inf = int(_pixel.CompOpType.CompOpInf)
    Sup = int(_pixel.CompOpType.CompOpSup)
    InfEqual = int(_pixel.CompOpType.CompOpInfEqual)
    SupEqual = int(_pixel.CompOpType.CompOpSupEqual)


# python/structuring_element/se_types.cpp
class se_type(enum.IntEnum):
    runtime = 0
    neighbor_list = 1
    image = 2
    chain = 3


class static_nl_se(enum.IntEnum):
    segx1d = int(Common_NL_SE.SESegmentX1D)
    square2d = int(Common_NL_SE.SESquare2D)
    cross2d = int(Common_NL_SE.SECross2D)
    segx2d = int(Common_NL_SE.SESegmentX2D)
    segy2d = int(Common_NL_SE.SESegmentY2D)
    segx3d = int(Common_NL_SE.SESegmentX3D)
    segy3d = int(Common_NL_SE.SESegmentY3D)
    segz3d = int(Common_NL_SE.SESegmentZ3D)
    cross3d = int(Common_NL_SE.SECross3D)
    square3d = int(Common_NL_SE.SESquare3D)


class static_compound_se(enum.IntEnum):
    octagon = int(Compound_NL_SE.Octagon)
    rhombicuboctahedron = int(Compound_NL_SE.Rhombicuboctahedron)


class RecType(enum.IntEnum):
    """python/geodesy/geodesy.cpp:14-17."""
    dilate = int(_geo.reconstruction_type.dilate)
    erode = int(_geo.reconstruction_type.erode)


# ----------------------------------------------------------------------------- images (python/base/image_interface.cpp)
class Image:
    """pypoutre.Image (poutre::IInterface) for a device image: a contiguous CUDA tensor, shared."""
    __slots__ = ("tensor",)

    def __init__(self, tensor: torch.Tensor):
        _image.descriptor(tensor, "Image")  # validates: CUDA, rank 1..3, contiguous, known pixel type
        self.tensor = tensor

    def ptype(self) -> PType:
        return PType(int(_image.GetPType(self.tensor)))

    def ctype(self) -> CType:
        return CType.Scalar

    def shape(self) -> list:
        return [int(s) for s in self.tensor.shape]

    def rank(self) -> int:
        return self.tensor.ndim

    def numpy(self) -> np.ndarray:
        """The pixels on the host (a device -> host copy)."""
        return self.tensor.cpu().numpy()

    def __dlpack__(self, **kwargs):
        return self.tensor.__dlpack__(**kwargs)

    def __dlpack_device__(self):
        return self.tensor.__dlpack_device__()

    def __repr__(self) -> str:  # image_t::str (image_t.hpp:118-131)
        tok = _image._TOKEN[_image.GetPType(self.tensor)]
        return (f"Image\n\tCtype: Scalar\n\tPtype: {tok}\n\tNumdim: {self.rank()}\n"
                f"\tcoord: ({', '.join(str(s) for s in self.shape())})\n")


def _t(img) -> torch.Tensor:
    """The device tensor behind an Image, a tensor, or a DLPack-exporting CUDA array (no copy)."""
    if isinstance(img, Image):
        return img.tensor
    if isinstance(img, torch.Tensor):
        return img
    if hasattr(img, "__dlpack__"):
        return torch.from_dlpack(img)
    raise TypeError(f"expected a device image, got {type(img).__name__}")


def _v(v):
    """A scalar operand (Python number or 0-d array) or an image operand."""
    if isinstance(v, (Image, torch.Tensor)) or (hasattr(v, "__dlpack__") and getattr(v, "ndim", 0) > 0):
        return _t(v)
    return v.item() if hasattr(v, "item") else v


def as_sizes_compatible(i_img1, i_img2) -> bool:
    return list(_t(i_img1).shape) == list(_t(i_img2).shape)


def as_types_compatible(i_img1, i_img2) -> bool:
    return _t(i_img1).dtype == _t(i_img2).dtype


def are_images_different(i_img1, i_img2) -> bool:
    """AreImagesDifferent (src/base/image_interface.cpp:52-56): distinct storage."""
    return _t(i_img1).data_ptr() != _t(i_img2).data_ptr()


def factory_image(shape, ctype=CType.Scalar, ptype=PType.GrayUINT8, device="cuda") -> Image:
    """poutre::Create(shape, ctype, ptype): a zero-filled device image."""
    if CType(ctype) != CType.Scalar:
        raise ValueError("only Scalar images are supported")
    return Image(_image.Create(shape, _image.PType(int(ptype)), device=device))


def from_string(s: str, device="cuda") -> Image:
    return Image(_image.ImageFromString(s, device=device))


def to_string(i_img) -> str:
    return _image.ImageToString(_t(i_img))


def from_numpy(a: np.ndarray, device="cuda") -> Image:
    """A device image holding a copy of the host array ``a``."""
    return Image(torch.from_numpy(np.ascontiguousarray(a)).to(device))


# ----------------------------------------------------------------------------- pixel processing
def arith_invert_image(i_img, o_img) -> None:
    _pixel.ArithInvertImage(_t(i_img), _t(o_img))


def arith_inf_image(i_img1, i_img2, o_img) -> None:
    _pixel.ArithInfImage(_t(i_img1), _t(i_img2), _t(o_img))


def arith_sup_image(i_img1, i_img2, o_img) -> None:
    _pixel.ArithSupImage(_t(i_img1), _t(i_img2), _t(o_img))


def arith_saturated_add_image(i_img1, i_img2, o_img) -> None:
    _pixel.ArithSaturatedAddImage(_t(i_img1), _t(i_img2), _t(o_img))


def arith_saturated_sub_image(i_img1, i_img2, o_img) -> None:
    _pixel.ArithSaturatedSubImage(_t(i_img1), _t(i_img2), _t(o_img))


def arith_saturated_add_constant(i_img, pvalue, o_img) -> None:
    _pixel.ArithSaturatedAddConstant(_t(i_img), pvalue, _t(o_img))


def arith_saturated_sub_constant(i_img, pvalue, o_img) -> None:
    _pixel.ArithSaturatedSubConstant(_t(i_img), pvalue, _t(o_img))


def compare(i_img, comp_op, i_comp, i_valtrue, i_valfalse, o_img) -> None:
    """The eight CompareImage overloads: each of comp / valtrue / valfalse a scalar or an image."""
    _pixel.CompareImage(_t(i_img), int(comp_op), _v(i_comp), _v(i_valtrue), _v(i_valfalse), _t(o_img))


def clone(i_img) -> Image:
    t = _t(i_img)
    o = torch.empty_like(t)
    _pixel.CopyInto(t, o)
    return Image(o)


def clone_geometry(i_img) -> Image:
    return Image(torch.empty_like(_t(i_img)))


def convert_geometry(i_img, ctype_or_ptype, ptype=None) -> Image:
    """ConvertGeometry(i, ctype, ptype) / ConvertGeometry(i, ptype): an image of that pixel type."""
    pt = ctype_or_ptype if ptype is None else ptype
    if ptype is not None and CType(ctype_or_ptype) != CType.Scalar:
        raise ValueError("only Scalar images are supported")
    t = _t(i_img)
    return Image(torch.empty(t.shape, dtype=_image.torch_dtype(_image.PType(int(pt))), device=t.device))


def convert(i_img, ctype, ptype) -> Image:
    o = convert_geometry(i_img, ctype, ptype)
    _pixel.ConvertInto(_t(i_img), o.tensor)
    return o


def copy_into(i_img, o_img) -> None:
    _pixel.CopyInto(_t(i_img), _t(o_img))


def convert_into(i_img, o_img) -> None:
    _pixel.ConvertInto(_t(i_img), _t(o_img))


# ----------------------------------------------------------------------------- low_level_morpho (python/low_level_morpho/ero_dil.cpp)
def _static_se(se):
    if isinstance(se, static_compound_se):
        return Compound_NL_SE(int(se))
    return Common_NL_SE(int(se))


def erode(i_img, se, iteration, o_img) -> None:
    """Erode(i, Common_NL_SE | Compound_NL_SE, iter | size, o)."""
    _llm.Erode(_t(i_img), _static_se(se), int(iteration), _t(o_img))


def dilate(i_img, se, iteration, o_img) -> None:
    _llm.Dilate(_t(i_img), _static_se(se), int(iteration), _t(o_img))


def dilateX(i_img, size_half_segment, o_img) -> None:
    _llm.DilateX(_t(i_img), int(size_half_segment), _t(o_img))


def dilateY(i_img, size_half_segment, o_img) -> None:
    _llm.DilateY(_t(i_img), int(size_half_segment), _t(o_img))


def erodeX(i_img, size_half_segment, o_img) -> None:
    _llm.ErodeX(_t(i_img), int(size_half_segment), _t(o_img))


def erodeY(i_img, size_half_segment, o_img) -> None:
    _llm.ErodeY(_t(i_img), int(size_half_segment), _t(o_img))


# ----------------------------------------------------------------------------- geodesy (python/geodesy/geodesy.cpp)
def reconstruction(rec_type, i_marker, i_mask, se, o_img) -> None:
    _geo.Reconstruction(_geo.reconstruction_type(int(rec_type)), _t(i_marker), _t(i_mask), Common_NL_SE(int(se)),
                        _t(o_img))


def h_minima(i_img, pvalue, se, o_img) -> None:
    _geo.h_minima(_t(i_img), pvalue, Common_NL_SE(int(se)), _t(o_img))


def h_maxima(i_img, pvalue, se, o_img) -> None:
    _geo.h_maxima(_t(i_img), pvalue, Common_NL_SE(int(se)), _t(o_img))


def h_concave(i_img, pvalue, se, o_img) -> None:
    _geo.h_concave(_t(i_img), pvalue, Common_NL_SE(int(se)), _t(o_img))


def h_convex(i_img, pvalue, se, o_img) -> None:
    _geo.h_convex(_t(i_img), pvalue, Common_NL_SE(int(se)), _t(o_img))


def dynamic_pseudo_closing(i_img, pvalue, se, o_img) -> None:
    _geo.dynamic_pseudo_closing(_t(i_img), pvalue, Common_NL_SE(int(se)), _t(o_img))


def dynamic_pseudo_opening(i_img, pvalue, se, o_img) -> None:
    _geo.dynamic_pseudo_opening(_t(i_img), pvalue, Common_NL_SE(int(se)), _t(o_img))


def high_leveling(i_ref, i_marker, se, o_img) -> None:
    _geo.high_leveling(_t(i_ref), _t(i_marker), Common_NL_SE(int(se)), _t(o_img))


def low_leveling(i_ref, i_marker, se, o_img) -> None:
    _geo.low_leveling(_t(i_ref), _t(i_marker), Common_NL_SE(int(se)), _t(o_img))


def leveling(i_ref, i_marker, se, o_img) -> None:
    _geo.leveling(_t(i_ref), _t(i_marker), Common_NL_SE(int(se)), _t(o_img))


# ----------------------------------------------------------------------------- label (python/label/label.cpp)
def label_binary(i_img, se, o_img) -> int:
    return _label.label_binary(_t(i_img), Common_NL_SE(int(se)), _t(o_img))


def label_flat_zones(i_img, se, o_img) -> int:
    return _label.label_flat_zones(_t(i_img), Common_NL_SE(int(se)), _t(o_img))


def label_maxima(i_img, se, o_img) -> None:
    _label.label_maxima(_t(i_img), Common_NL_SE(int(se)), _t(o_img))


def label_minima(i_img, se, o_img) -> None:
    _label.label_minima(_t(i_img), Common_NL_SE(int(se)), _t(o_img))
