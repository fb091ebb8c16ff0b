"""geodesy on device images, mirroring poutre2's public API (poutre::geo).

include/poutre/geodesy/mreconstruct.hpp:37-41, extrema.hpp:33-64, leveling.hpp:37-52.
The kernels run asynchronously on the current CUDA stream; with ``sync_checks`` on (the
default) each call then waits for its stream and raises ``PoutreError`` if the device gave
up (round cap / bounded wait), as the synchronous reference would throw.
"""
from __future__ import annotations

import ctypes
import enum
from typing import Sequence

import torch

from . import _lib
from .image import descriptor
from .se import Common_NL_SE

sync_checks = True


class reconstruction_type(enum.IntEnum):
    """poutre::geo::reconstruction_type (mreconstruct.hpp:28-31)."""
    erode = 0
    dilate = 1


def _stream():
    return _lib.current_stream()


def _post(check):
    if sync_checks if check is None else check:
        _lib.call("pg_check_device", _stream())


def Reconstruction(rect_type, i_marker, i_mask, nl_static, o_img, check=None):
    dm, dk, do = descriptor(i_marker, "marker"), descriptor(i_mask, "mask"), descriptor(o_img, "output")
    _lib.call("pg_reconstruction", int(reconstruction_type(rect_type)), ctypes.byref(dm), ctypes.byref(dk),
              int(Common_NL_SE(nl_static)), ctypes.byref(do), _stream())
    _post(check)


def _extrema(name, i_img, pvalue, nl_static, o_img, check):
    di, do = descriptor(i_img, "input"), descriptor(o_img, "output")
    h = _lib.scalar(di.ptype, pvalue)
    _lib.call(name, ctypes.byref(di), ctypes.byref(h), int(Common_NL_SE(nl_static)), ctypes.byref(do), _stream())
    _post(check)


def h_minima(i_img, pvalue, nl_static, o_img, check=None):
    _extrema("pg_h_minima", i_img, pvalue, nl_static, o_img, check)


def h_maxima(i_img, pvalue, nl_static, o_img, check=None):
    _extrema("pg_h_maxima", i_img, pvalue, nl_static, o_img, check)


def h_convex(i_img, pvalue, nl_static, o_img, check=None):
    _extrema("pg_h_convex", i_img, pvalue, nl_static, o_img, check)


def h_concave(i_img, pvalue, nl_static, o_img, check=None):
    _extrema("pg_h_concave", i_img, pvalue, nl_static, o_img, check)


def dynamic_pseudo_opening(i_img, pvalue, nl_static, o_img, check=None):
    _extrema("pg_dynamic_pseudo_opening", i_img, pvalue, nl_static, o_img, check)


def dynamic_pseudo_closing(i_img, pvalue, nl_static, o_img, check=None):
    _extrema("pg_dynamic_pseudo_closing", i_img, pvalue, nl_static, o_img, check)


def h_maxima_binary(i_img, pvalue, nl_static, o_img, check=None):
    """o_img (uint8) = 255 where i_img > h_maxima(i_img) else 0, one fused launch."""
    _extrema("pg_h_maxima_binary", i_img, pvalue, nl_static, o_img, check)


def h_maxima_binary_batch(imgs: Sequence[torch.Tensor], pvalue, nl_static, outs: Sequence[torch.Tensor], check=None):
    """Binary h-maxima of a ragged list of 2D images in one persistent launch."""
    n = len(imgs)
    if len(outs) != n:
        raise _lib.PoutreError(1, "h_maxima_binary_batch: as many outputs as inputs are needed")
    ins = (_lib.PgImage * n)(*[descriptor(t, "input") for t in imgs])
    ous = (_lib.PgImage * n)(*[descriptor(t, "output") for t in outs])
    h = _lib.scalar(ins[0].ptype if n else 4, pvalue)
    _lib.call("pg_h_maxima_binary_batch", ins, ous, n, ctypes.byref(h), int(Common_NL_SE(nl_static)), _stream())
    _post(check)


def _leveling(name, i_ref, i_marker, nl_static, o_img, check):
    dr, dm, do = descriptor(i_ref, "ref"), descriptor(i_marker, "marker"), descriptor(o_img, "output")
    _lib.call(name, ctypes.byref(dr), ctypes.byref(dm), int(Common_NL_SE(nl_static)), ctypes.byref(do), _stream())
    _post(check)


def low_leveling(i_ref, i_marker, nl_static, o_img, check=None):
    _leveling("pg_low_leveling", i_ref, i_marker, nl_static, o_img, check)


def high_leveling(i_ref, i_marker, nl_static, o_img, check=None):
    _leveling("pg_high_leveling", i_ref, i_marker, nl_static, o_img, check)


def leveling(i_ref, i_marker, nl_static, o_img, check=None):
    _leveling("pg_leveling", i_ref, i_marker, nl_static, o_img, check)


def last_reconstruction_rounds() -> int:
    return int(_lib.load().pg_last_reconstruction_rounds())


class HMaximaBinaryBatch:
    """Prepared ragged batch of the binary h-maxima (``pg_h_maxima_binary_batch_plan``).

    ``run()`` is one memset and one persistent launch over all images and can be captured in a
    CUDA graph.  With ``autotune`` the tile side and the sweep sets per tile visit are chosen by
    timing them on this batch (cached per pixel type, connectivity and size class).  The input
    and output tensors must stay alive and in place while the plan is used."""

    def __init__(self, imgs: Sequence[torch.Tensor], pvalue, nl_static, outs: Sequence[torch.Tensor],
                 autotune: bool = True):
        n = len(imgs)
        if len(outs) != n or n == 0:
            raise _lib.PoutreError(1, "HMaximaBinaryBatch: as many outputs as inputs (>= 1) are needed")
        self._keep = (list(imgs), list(outs))
        ins = (_lib.PgImage * n)(*[descriptor(t, "input") for t in imgs])
        ous = (_lib.PgImage * n)(*[descriptor(t, "output") for t in outs])
        self._plan = ctypes.c_void_p()
        h = _lib.scalar(ins[0].ptype, pvalue)
        _lib.call("pg_h_maxima_binary_batch_plan", ins, ous, n, ctypes.byref(h), int(Common_NL_SE(nl_static)),
                  int(bool(autotune)), ctypes.byref(self._plan), _stream())

    def run(self, check=False):
        _lib.call("pg_batch_plan_run", self._plan, _stream())
        _post(check)

    def set_config(self, tile: int, sweeps: int):
        """Pin the configuration instead of the autotuned one: tile 32 (register tiles) or 64
        (shared-memory tiles), sweep sets per tile visit >= 1."""
        _lib.call("pg_batch_plan_set_config", self._plan, int(tile), int(sweeps))

    @property
    def config(self):
        t, s, g = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _lib.call("pg_batch_plan_config", self._plan, ctypes.byref(t), ctypes.byref(s), ctypes.byref(g))
        return {"tile": t.value, "sweeps_per_visit": s.value, "grid": g.value}

    def close(self):
        if self._plan:
            _lib.load().pg_batch_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
