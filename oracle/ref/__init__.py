"""ctypes access to poutre2's own implementation (oracle/_ref/libpoutre_ref.so).

TEST INFRASTRUCTURE ONLY: used to cross-check the C restatement on random inputs and
as the timed CPU baseline.  ``available()`` is False when the library was not built
(poutre2 sources neither mounted nor staged)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .. import PTYPE, SE, OracleError

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(os.path.dirname(_HERE), "_ref", "libpoutre_ref.so")
_lib = None


def build():
    from . import build_ref
    return build_ref.build()


def available() -> bool:
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise OracleError("oracle/_ref/libpoutre_ref.so not built")
        L = ctypes.CDLL(LIB)
        P, I, I64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_erode_dilate_static.argtypes = [I, I, P, P, P, I, I, I]
        L.ref_erode_dilate_nl.argtypes = [I, I, P, P, P, P, I, I]
        L.ref_line.argtypes = [I, I, P, P, P, I64, I, I]
        L.ref_reconstruct.argtypes = [I, I, P, P, P, P, I, I]
        L.ref_extrema.argtypes = [I, I, I, P, P, P, D, I]
        L.ref_h_maxima_binary.argtypes = [I, P, P, P, D, I]
        L.ref_leveling.argtypes = [I, I, I, P, P, P, P, I]
        if hasattr(L, "ref_label"):
            L.ref_label.argtypes = [I, I, I, P, P, P, I, P]
        if hasattr(L, "ref_label_extrema"):
            L.ref_label_extrema.argtypes = [I, I, I, P, P, P, I]
        if hasattr(L, "ref_arith"):
            L.ref_arith.argtypes = [I, I, I, P, P, P, P]
            L.ref_compare.argtypes = [I, I, I, P, P, I, P, P, P]
            L.ref_convert.argtypes = [I, I, I, P, P, P]
        _lib = L
    return _lib


def _chk(rc):
    if rc != 0:
        raise OracleError("reference threw: " + lib().ref_last_error().decode())


def _shape(a):
    return (ctypes.c_int64 * 3)(*(list(a.shape) + [0] * (3 - a.ndim)))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def erode_dilate_static(img, se, iterations=1, dilate=True):
    a = np.ascontiguousarray(img); out = np.empty_like(a)
    _chk(lib().ref_erode_dilate_static(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), SE[se], iterations, int(dilate)))
    return out


def erode_dilate_compound(img, cse, size, dilate=True):
    """poutre::Erode/Dilate(i_img, Compound_NL_SE, size, o_img) on the compiled reference."""
    a = np.ascontiguousarray(img); out = np.empty_like(a)
    _chk(lib().ref_erode_dilate_compound(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out),
                                         {"Octagon": 1, "Rhombicuboctahedron": 2}[cse], int(size), int(dilate)))
    return out


def erode_dilate_nl(img, offsets, dilate=True):
    a = np.ascontiguousarray(img); out = np.empty_like(a)
    o = np.ascontiguousarray(np.array(offsets, dtype=np.int32).reshape(-1, a.ndim))
    _chk(lib().ref_erode_dilate_nl(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), _p(o), len(o), int(dilate)))
    return out


def line(img, half, axis="x", dilate=True):
    a = np.ascontiguousarray(img); out = np.empty_like(a)
    _chk(lib().ref_line(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), half, 0 if axis == "x" else 1, int(dilate)))
    return out


def reconstruct(marker, mask, se="SESquare2D", dilate=True):
    m = np.ascontiguousarray(marker); k = np.ascontiguousarray(mask); out = np.empty_like(m)
    _chk(lib().ref_reconstruct(PTYPE[m.dtype], m.ndim, _shape(m), _p(m), _p(k), _p(out), SE[se], int(dilate)))
    return out


_EXTREMA = ["h_minima", "h_maxima", "h_concave", "h_convex", "dynamic_pseudo_opening", "dynamic_pseudo_closing"]


def extrema(kind, img, h, se="SESquare2D"):
    a = np.ascontiguousarray(img); out = np.empty_like(a)
    _chk(lib().ref_extrema(_EXTREMA.index(kind), PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), float(h), SE[se]))
    return out


def h_maxima_binary(img, h, se="SESquare2D"):
    a = np.ascontiguousarray(img, dtype=np.uint8); out = np.empty_like(a)
    _chk(lib().ref_h_maxima_binary(a.ndim, _shape(a), _p(a), _p(out), float(h), SE[se]))
    return out


def leveling(kind, ref, marker, se="SESquare2D"):
    r = np.ascontiguousarray(ref); m = np.ascontiguousarray(marker); out = np.empty_like(r)
    k = {"low_leveling": 0, "high_leveling": 1, "leveling": 2}[kind]
    _chk(lib().ref_leveling(k, PTYPE[r.dtype], r.ndim, _shape(r), _p(r), _p(m), _p(out), SE[se]))
    return out


def label(img, se="SESquare2D", flat_zones=False):
    """poutre::label::label_binary / label_flat_zones on the compiled reference:
    returns (int64 label image, number of labels)."""
    a = np.ascontiguousarray(img)
    out = np.empty(a.shape, dtype=np.int64)
    n = ctypes.c_int64(0)
    _chk(lib().ref_label(int(flat_zones), PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), SE[se], ctypes.byref(n)))
    return out, int(n.value)


def label_extrema(img, se="SESquare2D", maxima=False):
    """poutre::label::label_minima / label_maxima on the compiled reference: the int64 label image."""
    a = np.ascontiguousarray(img)
    out = np.empty(a.shape, dtype=np.int64)
    _chk(lib().ref_label_extrema(int(maxima), PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), SE[se]))
    return out


ARITH = {"invert": 0, "sup": 1, "inf": 2, "sat_add": 3, "sat_sub": 4}


def arith(kind, a, b=None):
    """ArithInvert/Sup/Inf/SaturatedAdd/SaturatedSub image on the compiled reference."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(a if b is None else b)
    out = np.empty_like(a)
    _chk(lib().ref_arith(ARITH[kind], PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(b), _p(out)))
    return out


COMP = {"equal": 1, "diff": 2, "sup": 4, "sup_equal": 8, "inf": 16, "inf_equal": 32}


def compare(img, op, comp, valtrue, valfalse, out_dtype):
    """CompareImage on the compiled reference; each operand an ndarray (image) or a number (scalar)."""
    a = np.ascontiguousarray(img)
    od = np.dtype(out_dtype)
    out = np.empty(a.shape, dtype=od)
    keep, ptrs, vals = [], (ctypes.c_void_p * 3)(), (ctypes.c_double * 3)()
    for k, (v, dt) in enumerate(((comp, a.dtype), (valtrue, od), (valfalse, od))):
        if isinstance(v, np.ndarray):
            v = np.ascontiguousarray(v, dtype=dt)
            keep.append(v)
            ptrs[k] = v.ctypes.data
        else:
            vals[k] = float(v)
    _chk(lib().ref_compare(PTYPE[a.dtype], PTYPE[od], a.ndim, _shape(a), _p(a), COMP[op], ptrs, vals, _p(out)))
    return out


def convert(img, out_dtype):
    a = np.ascontiguousarray(img)
    out = np.empty(a.shape, dtype=np.dtype(out_dtype))
    _chk(lib().ref_convert(PTYPE[a.dtype], PTYPE[out.dtype], a.ndim, _shape(a), _p(a), _p(out)))
    return out
