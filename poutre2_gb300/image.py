"""Device images: the role of poutre::IInterface / image_t<T, Rank> on the GPU.

A device image is a contiguous CUDA ``torch.Tensor`` of rank 1..3 (row-major, last
dimension fastest, as image_t).  Helpers mirror poutre's base API:
``Create`` / ``Clone`` / ``CloneGeometry`` (src/base/image_interface.cpp,
src/pixel_processing/copy_convert.cpp:25,33), ``ImageFromString`` / ``ImageToString``
(include/poutre/base/image_interface.hpp:114-122), ``GetPType``.
"""
from __future__ import annotations

import enum

import numpy as np
import torch

from ._lib import PgImage, PoutreError


class PType(enum.IntEnum):
    """poutre::PType (include/poutre/base/types.hpp:517-526) + uint16."""
    PType_Undef = 0
    PType_GrayUINT8 = 4
    PType_GrayINT32 = 8
    PType_F32 = 16
    PType_GrayINT64 = 32
    PType_D64 = 64
    PType_GrayUINT16 = 128


_TORCH_TO_PTYPE = {
    torch.uint8: PType.PType_GrayUINT8,
    torch.int32: PType.PType_GrayINT32,
    torch.float32: PType.PType_F32,
    torch.int64: PType.PType_GrayINT64,
    torch.float64: PType.PType_D64,
    torch.uint16: PType.PType_GrayUINT16,
}
_PTYPE_TO_TORCH = {v: k for k, v in _TORCH_TO_PTYPE.items()}
_TOKEN = {PType.PType_GrayUINT8: "GUINT8", PType.PType_GrayINT32: "GINT32", PType.PType_GrayINT64: "GINT64",
          PType.PType_F32: "F32", PType.PType_D64: "D64", PType.PType_GrayUINT16: "GUINT16"}
_FROM_TOKEN = {v: k for k, v in _TOKEN.items()}
_NP = {PType.PType_GrayUINT8: np.uint8, PType.PType_GrayINT32: np.int32, PType.PType_GrayINT64: np.int64,
       PType.PType_F32: np.float32, PType.PType_D64: np.float64, PType.PType_GrayUINT16: np.uint16}


def GetPType(img: torch.Tensor) -> PType:
    try:
        return _TORCH_TO_PTYPE[img.dtype]
    except KeyError:
        raise PoutreError(2, f"unsupported PTYPE {img.dtype}") from None


def torch_dtype(ptype) -> torch.dtype:
    return _PTYPE_TO_TORCH[PType(ptype)]


def numpy_dtype(ptype):
    return _NP[PType(ptype)]


def _require_device_image(img: torch.Tensor, what: str):
    if not isinstance(img, torch.Tensor):
        raise PoutreError(1, f"{what}: expected a torch.Tensor device image")
    if not img.is_cuda:
        raise PoutreError(7, f"{what}: image must live on a CUDA device (no CPU path)")
    if img.ndim < 1 or img.ndim > 3:
        raise PoutreError(1, f"{what}: unsupported number of dims:{img.ndim}")
    if not img.is_contiguous():
        raise PoutreError(1, f"{what}: image must be contiguous (row-major)")


def descriptor(img: torch.Tensor, what: str = "image") -> PgImage:
    """pg_image descriptor of a contiguous CUDA tensor."""
    _require_device_image(img, what)
    d = PgImage()
    d.data = img.data_ptr()
    d.ptype = int(GetPType(img))
    d.rank = img.ndim
    for i, s in enumerate(img.shape):
        d.shape[i] = int(s)
    return d


def Create(dims, ptype, device="cuda") -> torch.Tensor:
    """poutre::Create(dims, CompoundType_Scalar, ptype) on the device."""
    return torch.zeros(tuple(int(d) for d in dims), dtype=torch_dtype(ptype), device=device)


def Clone(img: torch.Tensor) -> torch.Tensor:
    return img.clone()


def CloneGeometry(img: torch.Tensor) -> torch.Tensor:
    return torch.empty_like(img)


def ImageFromString(s: str, device="cuda") -> torch.Tensor:
    """Parse poutre's image string ``"Scalar <PTYPE> <rank> <d0..> <values..>"``; reads exactly
    prod(shape) values and ignores trailing tokens, as the reference (image_interface.cpp:407-425)."""
    toks = s.replace("\\\n", " ").split()
    if not toks or toks[0] != "Scalar":
        raise PoutreError(1, "ImageFromString: only Scalar images are supported")
    pt = _FROM_TOKEN[toks[1]]
    rank = int(toks[2])
    shape = [int(t) for t in toks[3:3 + rank]]
    n = int(np.prod(shape)) if shape else 0
    vals = toks[3 + rank:3 + rank + n]
    if len(vals) < n:
        raise PoutreError(1, "ImageFromString: unable to read current pixel")
    conv = float if pt in (PType.PType_F32, PType.PType_D64) else int
    arr = np.array([conv(v) for v in vals], dtype=_NP[pt]).reshape(shape)
    return torch.from_numpy(arr).to(device)


def ImageToString(img: torch.Tensor) -> str:
    pt = GetPType(img)
    a = img.detach().cpu().numpy().reshape(-1)
    head = ["Scalar", _TOKEN[pt], str(img.ndim)] + [str(int(s)) for s in img.shape]
    if pt in (PType.PType_F32, PType.PType_D64):
        body = [repr(float(v)) for v in a]
    else:
        body = [str(int(v)) for v in a]
    return " ".join(head + body)
