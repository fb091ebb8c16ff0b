"""ctypes binding of ``_build/libpoutre_gb300.so`` (the C ABI of ``include/poutre_gb300.h``).

The library is the only compute path.  Loading fails loudly (``PoutreError``) when it has
not been built or when no CUDA device is present; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libpoutre_gb300.so")

PG_OK = 0
STATUS_NAMES = {
    0: "PG_OK", 1: "PG_ERR_INVALID_ARGUMENT", 2: "PG_ERR_UNSUPPORTED_PTYPE", 3: "PG_ERR_UNSUPPORTED_SE",
    4: "PG_ERR_INCOMPATIBLE", 5: "PG_ERR_ALIASING", 6: "PG_ERR_NOT_SQUARE", 7: "PG_ERR_CUDA",
    8: "PG_ERR_OUT_OF_MEMORY", 9: "PG_ERR_NOT_CONVERGED", 10: "PG_ERR_SCALAR_TYPE",
}

# every symbol include/poutre_gb300.h declares
EXPORTED = [
    "pg_last_error", "pg_version",
    "pg_erode", "pg_dilate", "pg_erode_compound", "pg_dilate_compound", "pg_erode_nl", "pg_dilate_nl",
    "pg_erode_x", "pg_dilate_x", "pg_erode_y", "pg_dilate_y",
    "pg_erode_se", "pg_dilate_se", "pg_opening", "pg_closing", "pg_gradient",
    "pg_label_binary", "pg_label_flat_zones", "pg_label_minima", "pg_label_maxima",
    "pg_reconstruction", "pg_h_minima", "pg_h_maxima", "pg_h_concave", "pg_h_convex",
    "pg_dynamic_pseudo_opening", "pg_dynamic_pseudo_closing", "pg_h_maxima_binary", "pg_h_maxima_binary_batch",
    "pg_low_leveling", "pg_high_leveling", "pg_leveling",
    "pg_sat_sub_constant", "pg_sat_add_constant",
    "pg_arith_invert_image", "pg_arith_sup_image", "pg_arith_inf_image", "pg_sat_add_image", "pg_sat_sub_image",
    "pg_compare_image", "pg_copy_into", "pg_convert_into",
    "pg_flat_morph2d_forward", "pg_flat_morph2d_backward", "pg_flat_morph2d_forward_arg",
    "pg_flat_morph2d_backward_arg",
    "pg_check_device", "pg_last_reconstruction_rounds", "pg_reconstruction_noalloc",
    "pg_h_maxima_binary_batch_plan", "pg_batch_plan_run", "pg_batch_plan_config", "pg_batch_plan_set_config",
    "pg_batch_plan_destroy", "pg_debug_set_limits", "pg_debug_fail_allocations",
]


class PoutreError(RuntimeError):
    """Raised where poutre2 throws std::runtime_error (the C ABI returned a non-zero status)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class PgImage(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("ptype", ctypes.c_int32), ("rank", ctypes.c_int32),
                ("shape", ctypes.c_int64 * 3)]


class _ScalarValue(ctypes.Union):
    _fields_ = [("u8", ctypes.c_uint8), ("u16", ctypes.c_uint16), ("i32", ctypes.c_int32), ("i64", ctypes.c_int64),
                ("f32", ctypes.c_float), ("f64", ctypes.c_double)]


class PgScalar(ctypes.Structure):
    """pg_scalar: one pixel value held exactly, tagged with its pixel type (ScalarTypeVariant)."""
    _fields_ = [("ptype", ctypes.c_int32), ("reserved_", ctypes.c_int32), ("v", _ScalarValue)]


# pg_ptype -> (union member, lowest, highest); floating-point members have no bounds here
_SCALAR_MEMBER = {4: ("u8", 0, 255), 128: ("u16", 0, 65535), 8: ("i32", -2**31, 2**31 - 1),
                  32: ("i64", -2**63, 2**63 - 1), 16: ("f32", None, None), 64: ("f64", None, None)}
_NUMPY_PTYPE = {"uint8": 4, "uint16": 128, "int32": 8, "int64": 32, "float32": 16, "float64": 64}


def scalar(ptype: int, value) -> PgScalar:
    """The pg_scalar a call receives for `value`.

    A numpy scalar keeps its own type (``np.int32(5)`` holds INT32), and the library then checks it
    against the pixel type as poutre2's ``std::get`` checks a ScalarTypeVariant (PG_ERR_SCALAR_TYPE
    on a mismatch).  A Python int or float is taken as pixel type `ptype`: an integer type needs an
    integral value in its range (Python ints stay exact up to the int64 limits), else
    PoutreError(PG_ERR_SCALAR_TYPE) is raised here."""
    import numbers

    import numpy as np
    if isinstance(value, np.generic):
        pt = _NUMPY_PTYPE.get(value.dtype.name)
        if pt is None:
            raise PoutreError(10, f"no pixel type holds a {value.dtype.name} scalar")
        value = value.item()
    else:
        pt = int(ptype)
    if pt not in _SCALAR_MEMBER:
        raise PoutreError(2, f"unsupported PTYPE {pt}")
    member, lo, hi = _SCALAR_MEMBER[pt]
    s = PgScalar()
    s.ptype = pt
    if lo is None:
        if isinstance(value, bool) or not isinstance(value, numbers.Real):
            raise PoutreError(10, f"{value!r} is not a value of a floating-point pixel type")
        setattr(s.v, member, float(value))
        return s
    if isinstance(value, float) and value.is_integer():
        value = int(value)
    if isinstance(value, bool) or not isinstance(value, numbers.Integral) or not lo <= int(value) <= hi:
        raise PoutreError(10, f"{value!r} is not a value of the pixel type ({member})")
    setattr(s.v, member, int(value))
    return s


class PgOperand(ctypes.Structure):
    """pg_operand: an image (``image`` set) or the scalar ``value`` of CompareImage."""
    _fields_ = [("image", ctypes.POINTER(PgImage)), ("value", PgScalar)]


class PgSE(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("common_se", ctypes.c_int32), ("iter", ctypes.c_int32),
                ("hy", ctypes.c_int32), ("hx", ctypes.c_int32), ("dy", ctypes.c_int32), ("dx", ctypes.c_int32),
                ("half", ctypes.c_int32), ("offsets", ctypes.POINTER(ctypes.c_int32)), ("n", ctypes.c_int32)]


_lock = threading.Lock()
_lib = None


def load(path: str | None = None):
    """Load the library (once).  Raises PoutreError if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise PoutreError(7, f"CUDA library not built: {p} (run __graft_entry__.build())")
        L = ctypes.CDLL(p)
        img = ctypes.POINTER(PgImage)
        se = ctypes.POINTER(PgSE)
        I32, I64, VP = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
        i32p = ctypes.POINTER(ctypes.c_int32)
        fp = ctypes.c_void_p
        D = ctypes.POINTER(PgScalar)  # the scalar arguments (h, v): const pg_scalar *
        sig = {
            "pg_erode": [img, I32, I32, img, VP], "pg_dilate": [img, I32, I32, img, VP],
            "pg_erode_compound": [img, I32, I32, img, VP], "pg_dilate_compound": [img, I32, I32, img, VP],
            "pg_erode_nl": [img, i32p, I32, img, VP], "pg_dilate_nl": [img, i32p, I32, img, VP],
            "pg_erode_x": [img, I64, img, VP], "pg_dilate_x": [img, I64, img, VP],
            "pg_erode_y": [img, I64, img, VP], "pg_dilate_y": [img, I64, img, VP],
            "pg_erode_se": [img, se, img, VP], "pg_dilate_se": [img, se, img, VP],
            "pg_opening": [img, se, img, VP], "pg_closing": [img, se, img, VP], "pg_gradient": [img, se, img, VP],
            "pg_label_binary": [img, I32, img, ctypes.POINTER(I64), VP],
            "pg_label_flat_zones": [img, I32, img, ctypes.POINTER(I64), VP],
            "pg_label_minima": [img, I32, img, ctypes.POINTER(I64), VP],
            "pg_label_maxima": [img, I32, img, ctypes.POINTER(I64), VP],
            "pg_reconstruction": [I32, img, img, I32, img, VP],
            "pg_h_minima": [img, D, I32, img, VP], "pg_h_maxima": [img, D, I32, img, VP],
            "pg_h_concave": [img, D, I32, img, VP], "pg_h_convex": [img, D, I32, img, VP],
            "pg_dynamic_pseudo_opening": [img, D, I32, img, VP], "pg_dynamic_pseudo_closing": [img, D, I32, img, VP],
            "pg_h_maxima_binary": [img, D, I32, img, VP],
            "pg_h_maxima_binary_batch": [img, img, I32, D, I32, VP],
            "pg_low_leveling": [img, img, I32, img, VP], "pg_high_leveling": [img, img, I32, img, VP],
            "pg_leveling": [img, img, I32, img, VP],
            "pg_sat_sub_constant": [img, D, img, VP], "pg_sat_add_constant": [img, D, img, VP],
            "pg_arith_invert_image": [img, img, VP], "pg_arith_sup_image": [img, img, img, VP],
            "pg_arith_inf_image": [img, img, img, VP], "pg_sat_add_image": [img, img, img, VP],
            "pg_sat_sub_image": [img, img, img, VP],
            "pg_compare_image": [img, I32, ctypes.POINTER(PgOperand), ctypes.POINTER(PgOperand),
                                 ctypes.POINTER(PgOperand), img, VP],
            "pg_copy_into": [img, img, VP], "pg_convert_into": [img, img, VP],
            "pg_flat_morph2d_forward": [fp, fp, I64, I64, I64, I32, I32, I32, VP],
            "pg_flat_morph2d_backward": [fp, fp, fp, I64, I64, I64, I32, I32, I32, VP],
            "pg_flat_morph2d_forward_arg": [fp, fp, VP, I64, I64, I64, I32, I32, VP],
            "pg_flat_morph2d_backward_arg": [VP, fp, fp, I64, I64, I64, I32, VP],
            "pg_check_device": [VP],
            "pg_reconstruction_noalloc": [I32, img, img, I32, img, VP],
            "pg_h_maxima_binary_batch_plan": [img, img, I32, D, I32, I32, ctypes.POINTER(VP), VP],
            "pg_batch_plan_run": [VP, VP],
            "pg_batch_plan_config": [VP, ctypes.POINTER(I32), ctypes.POINTER(I32), ctypes.POINTER(I32)],
            "pg_batch_plan_set_config": [VP, I32, I32],
            "pg_batch_plan_destroy": [VP],
            "pg_debug_set_limits": [I32, I64], "pg_debug_fail_allocations": [I32],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.pg_last_error.restype = ctypes.c_char_p
        L.pg_last_error.argtypes = []
        L.pg_version.restype = ctypes.c_char_p
        L.pg_version.argtypes = []
        L.pg_last_reconstruction_rounds.restype = ctypes.c_int32
        L.pg_last_reconstruction_rounds.argtypes = []
        _lib = L
        return L


def current_stream() -> ctypes.c_void_p:
    """The current CUDA stream of the current device as a cudaStream_t (the stream every call is
    queued on).  Reads the raw handle directly where torch exposes it (building a torch Stream object
    costs about 3 us a call), else through torch.cuda.current_stream()."""
    import torch
    raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if raw is not None:
        return ctypes.c_void_p(raw(torch.cuda.current_device()))
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def check(status: int):
    if status != PG_OK:
        raise PoutreError(status, load().pg_last_error().decode(errors="replace"))


def call(name: str, *args):
    check(getattr(load(), name)(*args))
