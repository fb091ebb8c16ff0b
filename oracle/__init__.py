"""CPU oracle for the poutre2 morphology + geodesy hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package, and only as the checker.
The product (``poutre2_gb300``) never imports it.

The heavy routines live in ``poutre_oracle.c`` (plain C restatement of the
reference algorithms, each citing the poutre2 file:line it follows).  The
pointwise glue (saturated arithmetic, comparisons) and the compositions the
reference builds from them (h-extrema, dynamic pseudo opening/closing,
leveling) are restated here in numpy, again citing the reference.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD_DIR, "libpoutre_oracle.so")
_SRC = os.path.join(_HERE, "poutre_oracle.c")

# poutre::PType values (include/poutre/base/types.hpp:517-526) + 128 for uint16.
PTYPE = {
    np.dtype(np.uint8): 4,
    np.dtype(np.int32): 8,
    np.dtype(np.float32): 16,
    np.dtype(np.int64): 32,
    np.dtype(np.float64): 64,
    np.dtype(np.uint16): 128,
}

# poutre::se::Common_NL_SE (include/poutre/structuring_element/se_types_and_tags.hpp:45-57)
SE = {
    "SESegmentX1D": 1, "SESquare2D": 2, "SECross2D": 3, "SESegmentX2D": 4, "SESegmentY2D": 5,
    "SESegmentX3D": 6, "SESegmentY3D": 7, "SESegmentZ3D": 8, "SECross3D": 9, "SESquare3D": 10,
}

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile poutre_oracle.c into oracle/_build/libpoutre_oracle.so (gcc, -O2)."""
    os.makedirs(_BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", _SRC, "-o", tmp])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            P, I, I64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
            L.or_erode_dilate_nl.argtypes = [I, I, P, P, P, P, I, I]
            L.or_erode_dilate_static.argtypes = [I, I, P, P, P, I, I, I]
            L.or_line.argtypes = [I, I, P, P, P, I64, I, I]
            L.or_reconstruct.argtypes = [I, I, P, P, P, P, I, I]
            L.or_leveling_half.argtypes = [I, I, P, P, P, P, I, I]
            L.or_flat2d_forward.argtypes = [I64, I64, I64, P, P, I, I, I]
            L.or_flat2d_backward.argtypes = [I64, I64, I64, P, P, P, I, I, I]
            L.or_label.argtypes = [I, I, P, P, P, I, I, P]
            _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _check(rc: int, what: str):
    if rc != 0:
        raise OracleError(f"{what}: oracle rejected the call (code {rc})")


def _shape(a: np.ndarray):
    s = (ctypes.c_int64 * 3)(*(list(a.shape) + [0] * (3 - a.ndim)))
    return s


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a) -> np.ndarray:
    a = np.ascontiguousarray(a)
    if a.dtype not in PTYPE:
        raise OracleError(f"unsupported dtype {a.dtype}")
    return a


# ----------------------------------------------------------------------------- low level morpho
def erode_dilate_static(img, se: str, iterations: int = 1, dilate: bool = True) -> np.ndarray:
    """poutre::Erode/Dilate(i_img, Common_NL_SE, iter, o_img)
    (src/low_level_morpho/ero_dil_static.cpp:229-306)."""
    a = _c(img)
    out = np.empty_like(a)
    _check(lib().or_erode_dilate_static(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), SE[se],
                                        int(iterations), int(dilate)), f"{'Dilate' if dilate else 'Erode'}({se})")
    return out


def dilate(img, se: str = "SESquare2D", iterations: int = 1):
    return erode_dilate_static(img, se, iterations, True)


def erode(img, se: str = "SESquare2D", iterations: int = 1):
    return erode_dilate_static(img, se, iterations, False)


def compound_passes(cse: str, size: int):
    """The passes of t_DilateOctagon / t_DilateRhombicuboctahedron
    (low_level_morpho/details/ero_dil_compound_static_se_t.hpp:34-95): `size` passes, the last
    round(size / (1 + sqrt 2)) (halves rounded up) by the square, the others by the cross."""
    cross, square = ("SECross2D", "SESquare2D") if cse == "Octagon" else ("SECross3D", "SESquare3D")
    if size <= 0:
        return []
    if size == 1:
        return ["SECross2D"]  # the reference's size-1 case uses the 2D cross for both
    nb = size / (1 + np.sqrt(2.0))
    nsq = int(np.floor(nb) if nb - np.floor(nb) < 0.5 else np.floor(nb) + 1)
    return [cross] * (size - nsq) + [square] * nsq


def erode_dilate_compound(img, cse: str, size: int, dilate: bool = True) -> np.ndarray:
    """poutre::Erode/Dilate(i_img, Compound_NL_SE, size, o_img) (src/low_level_morpho/ero_dil_compound_static.cpp):
    the static passes of compound_passes() in order."""
    a = _c(img).copy()
    for se in compound_passes(cse, size):
        a = erode_dilate_static(a, se, 1, dilate)
    return a


def erode_dilate_nl(img, offsets, dilate: bool = True) -> np.ndarray:
    """poutre::Erode/Dilate(i_img, IStructuringElement, o_img) with a neighbour list
    (src/low_level_morpho/ero_dil.cpp:59,152; ero_dil_runtime_nl_se_t.hpp:54-96).
    ``offsets``: tuples in reference order (d0..d_rank-1)."""
    a = _c(img)
    out = np.empty_like(a)
    trip = []
    for o in offsets:
        o = tuple(int(v) for v in o)
        if len(o) != a.ndim:
            raise OracleError("offset rank differs from image rank")
        trip.append((0,) * (3 - a.ndim) + o)
    arr = np.ascontiguousarray(np.array(trip, dtype=np.int32).reshape(-1, 3))
    _check(lib().or_erode_dilate_nl(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), _p(arr), len(trip),
                                    int(dilate)), "Erode/Dilate(neighbor list)")
    return out


def line(img, half: int, axis: str = "x", dilate: bool = True) -> np.ndarray:
    """poutre::DilateX/ErodeX/DilateY/ErodeY (src/low_level_morpho/ero_dil_line.cpp:80,144,189,252)."""
    a = _c(img)
    out = np.empty_like(a)
    _check(lib().or_line(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), int(half), 0 if axis == "x" else 1,
                         int(dilate)), f"line {axis}")
    return out


def segment_offsets(dy: int, dx: int, half: int, rank: int = 2):
    """Offsets t*(dy,dx), t in [-half, half], centre first (runtime neighbour list)."""
    offs = [(0, 0)] + [(t * dy, t * dx) for t in range(-half, half + 1) if t != 0]
    return offs


# ----------------------------------------------------------------------------- pixel processing
def _limits(dt):
    """TypeTraits<T>::min()/max() for the integer types (types_traits.hpp:109-265)."""
    return np.iinfo(dt).min, np.iinfo(dt).max


def _saturate(a, b, add: bool):
    """Saturated a + b / a - b of one pixel type: for integer pixels the exact sum or difference
    clamped to [TypeTraits<T>::min(), max()] (xsimd's sadd / ssub, which the reference's vector body
    applies; its scalar remainder loop agrees on every result that is in range of its accumulator),
    for floating-point pixels the plain IEEE sum or difference of that vector body."""
    if np.issubdtype(a.dtype, np.integer):
        lo, hi = _limits(a.dtype)
        wide = object if a.dtype.itemsize == 8 else np.int64   # exact for 64-bit pixels too
        r = a.astype(wide) + b.astype(wide) if add else a.astype(wide) - b.astype(wide)
        return np.clip(r, lo, hi).astype(a.dtype)
    return (a + b if add else a - b).astype(a.dtype)


def sat_sub_const(img, h):
    """ArithSaturatedSubConstant (src/pixel_processing/arith.cpp:471; op_Saturated_Sub_Constant
    arith_op_t.hpp:281-345)."""
    a = _c(img)
    return _saturate(a, np.asarray(h).astype(a.dtype), False)


def sat_add_const(img, h):
    """ArithSaturatedAddConstant (op_Saturated_Add_Constant, arith_op_t.hpp:218-276)."""
    a = _c(img)
    return _saturate(a, np.asarray(h).astype(a.dtype), True)


def sat_sub_image(a, b):
    """ArithSaturatedSubImage (src/pixel_processing/arith.cpp:195; op_Saturated_Sub arith_op_t.hpp:84-121)."""
    return _saturate(_c(a), _c(b), False)


def sat_add_image(a, b):
    """ArithSaturatedAddImage (src/pixel_processing/arith.cpp:125; op_Saturated_Add arith_op_t.hpp:146-183)."""
    return _saturate(_c(a), _c(b), True)


def sup_image(a, b):
    """ArithSupImage (op_Sup arith_op_t.hpp:346-366): a > b ? a : b."""
    a = _c(a); b = _c(b)
    return np.where(a > b, a, b).astype(a.dtype)


def inf_image(a, b):
    """ArithInfImage (op_Inf arith_op_t.hpp:396-417): a < b ? a : b."""
    a = _c(a); b = _c(b)
    return np.where(a < b, a, b).astype(a.dtype)


def invert_image(a):
    """ArithInvertImage (op_Invert arith_op_t.hpp:40-58): -a in the pixel type (wraps for unsigned
    and for the most negative signed value)."""
    a = _c(a)
    with np.errstate(over="ignore"):
        return np.negative(a).astype(a.dtype)


COMPARE_OPS = {"equal": np.equal, "diff": np.not_equal, "sup": np.greater, "sup_equal": np.greater_equal,
               "inf": np.less, "inf_equal": np.less_equal}


def compare(img, op: str, comp, valtrue, valfalse, out_dtype):
    """CompareImage (include/poutre/pixel_processing/compare.hpp:31-84; OpComp* compare_op_t.hpp:41-165):
    out = op(img, comp) ? valtrue : valfalse.  comp (a scalar or an image) has the input's type,
    valtrue / valfalse (scalars or images) the output's."""
    a = _c(img)
    od = np.dtype(out_dtype)
    c = np.asarray(comp).astype(a.dtype)
    t = np.asarray(valtrue).astype(od)
    f = np.asarray(valfalse).astype(od)
    return np.where(COMPARE_OPS[op](a, c), t, f).astype(od)


def convert(img, out_dtype):
    """ConvertInto (src/pixel_processing/copy_convert.cpp:301; CopyOpDispatcher copy_convert_t.hpp:33-86):
    static_cast of every pixel (truncation toward zero from floating point, modular narrowing of
    integers, round-to-nearest into floating point); defined for values the target type holds."""
    return _c(img).astype(np.dtype(out_dtype))


def lowest(dt):
    dt = np.dtype(dt)
    return np.iinfo(dt).min if np.issubdtype(dt, np.integer) else np.finfo(dt).min


def highest(dt):
    dt = np.dtype(dt)
    return np.iinfo(dt).max if np.issubdtype(dt, np.integer) else np.finfo(dt).max


# ----------------------------------------------------------------------------- geodesy
def reconstruct(marker, mask, se: str = "SESquare2D", dilate: bool = True) -> np.ndarray:
    """poutre::geo::Reconstruction (src/geodesy/mreconstruct.cpp:48-133)."""
    m = _c(marker); k = _c(mask)
    if m.dtype != k.dtype or m.shape != k.shape:
        raise OracleError("marker/mask mismatch")
    out = np.empty_like(m)
    _check(lib().or_reconstruct(PTYPE[m.dtype], m.ndim, _shape(m), _p(m), _p(k), _p(out), SE[se], int(dilate)),
           "Reconstruction")
    return out


def h_maxima(img, h, se="SESquare2D"):
    """src/geodesy/extrema.cpp:39-49: Rec_dilate(sat_sub(f, h), f)."""
    return reconstruct(sat_sub_const(img, h), img, se, True)


def h_minima(img, h, se="SESquare2D"):
    """src/geodesy/extrema.cpp:27-37: Rec_erode(sat_add(f, h), f)."""
    return reconstruct(sat_add_const(img, h), img, se, False)


def h_convex(img, h, se="SESquare2D"):
    """src/geodesy/extrema.cpp:63-73: sat_sub(f, h_maxima(f))."""
    return sat_sub_image(img, h_maxima(img, h, se))


def h_concave(img, h, se="SESquare2D"):
    """src/geodesy/extrema.cpp:51-61: sat_sub(h_minima(f), f)."""
    return sat_sub_image(h_minima(img, h, se), img)


def dynamic_pseudo_opening(img, h, se="SESquare2D"):
    """src/geodesy/extrema.cpp:75-93."""
    f = _c(img)
    tmp = sat_sub_const(f, h)
    ext = reconstruct(tmp, f, se, True)
    lo = f.dtype.type(lowest(f.dtype))
    mask = np.where(ext == tmp, f, lo).astype(f.dtype)          # CompareImage(ext, Equal, tmp, f, lowest)
    tmp2 = np.where(ext != lo, mask, lo).astype(f.dtype)        # CompareImage(ext, Diff, lowest, mask, lowest)
    return reconstruct(tmp2, f, se, True)


def dynamic_pseudo_closing(img, h, se="SESquare2D"):
    """src/geodesy/extrema.cpp:95-114."""
    f = _c(img)
    tmp = sat_add_const(f, h)
    ext = reconstruct(tmp, f, se, False)
    hi = f.dtype.type(highest(f.dtype))
    mask = np.where(ext == tmp, f, hi).astype(f.dtype)
    tmp2 = np.where(ext != hi, mask, hi).astype(f.dtype)
    return reconstruct(tmp2, f, se, False)


def h_maxima_binary(img, h, se="SESquare2D"):
    """Binary regional maxima of the h-maxima transform:
    CompareImage(f, CompOpSup, h_maxima(f), 255, 0) (compare.hpp:69 overload)."""
    f = _c(img)
    rec = h_maxima(f, h, se)
    return np.where(f > rec, 255, 0).astype(np.uint8)


def low_leveling(ref, marker, se="SESquare2D"):
    r = _c(ref); m = _c(marker)
    out = np.empty_like(m)
    _check(lib().or_leveling_half(PTYPE[r.dtype], r.ndim, _shape(r), _p(r), _p(m), _p(out), SE[se], 1), "low_leveling")
    return out


def high_leveling(ref, marker, se="SESquare2D"):
    r = _c(ref); m = _c(marker)
    out = np.empty_like(m)
    _check(lib().or_leveling_half(PTYPE[r.dtype], r.ndim, _shape(r), _p(r), _p(m), _p(out), SE[se], 0), "high_leveling")
    return out


def leveling(ref, marker, se="SESquare2D"):
    """src/geodesy/leveling.cpp:231-238: low_leveling(high_leveling(ref, marker), marker)."""
    return low_leveling(high_leveling(ref, marker, se), marker, se)


# ----------------------------------------------------------------------------- composites (no reference counterpart)
def opening_static(img, se, iterations=1):
    return dilate(erode(img, se, iterations), se, iterations)


def closing_static(img, se, iterations=1):
    return erode(dilate(img, se, iterations), se, iterations)


def gradient_from(dil, ero):
    """Plain subtraction dilate - erode (never the saturated op: for f32 its scalar path clamps
    at FLT_MIN, arith_op_t.hpp:281-345)."""
    return (dil - ero).astype(dil.dtype)


def line_y_any(img, half: int, dilate: bool = True) -> np.ndarray:
    """Vertical running min/max of any 2D image: the X restatement on the transposed image.
    (The reference's DilateY only accepts square images; the window itself does not care.)"""
    a = _c(img)
    return np.ascontiguousarray(line(np.ascontiguousarray(a.T), half, "x", dilate).T)


def rect(img, hy, hx, dilate=True):
    """Flat (2hy+1)x(2hx+1) rectangle = Y(hy) o X(hx) running min/max; equals the reference's
    DilateY(DilateX(.)) and Dilate(SESquare2D, iter=h) for hy == hx == h."""
    t = line(img, hx, "x", dilate) if hx > 0 else _c(img).copy()
    return line_y_any(t, hy, dilate) if hy > 0 else t


# ----------------------------------------------------------------------------- labelling
def label(img, se: str = "SESquare2D", flat_zones: bool = False):
    """poutre::label::label_binary / label_flat_zones(i_img, Common_NL_SE, o_img)
    (src/label/label_binary.cpp, label_flat_zones.cpp; include/poutre/label/details/label_t.hpp:132-247):
    returns (int64 label image, number of labels)."""
    a = _c(img)
    out = np.empty(a.shape, dtype=np.int64)
    count = ctypes.c_int64(0)
    _check(lib().or_label(PTYPE[a.dtype], a.ndim, _shape(a), _p(a), _p(out), SE[se], int(flat_zones),
                          ctypes.byref(count)), f"label_{'flat_zones' if flat_zones else 'binary'}({se})")
    return out, int(count.value)


def label_extrema(img, se: str = "SESquare2D", maxima: bool = False):
    """poutre::label::label_minima / label_maxima (src/label/label_extrema.cpp): label_binary of
    h_concave(f, 1) / h_convex(f, 1); returns (int64 label image, number of labels)."""
    ext = h_convex(img, 1, se) if maxima else h_concave(img, 1, se)
    return label(ext, se)


# ----------------------------------------------------------------------------- adjoint
def flat2d_forward(x, r: int, dilate: bool):
    a = np.ascontiguousarray(x, dtype=np.float32)
    H, W = a.shape[-2:]
    planes = a.size // (H * W)
    out = np.empty_like(a)
    lib().or_flat2d_forward(planes, H, W, _p(a), _p(out), r, r, int(dilate))
    return out


def flat2d_backward(x, gout, r: int, dilate: bool):
    a = np.ascontiguousarray(x, dtype=np.float32)
    g = np.ascontiguousarray(gout, dtype=np.float32)
    H, W = a.shape[-2:]
    planes = a.size // (H * W)
    gin = np.empty_like(a)
    lib().or_flat2d_backward(planes, H, W, _p(a), _p(g), _p(gin), r, r, int(dilate))
    return gin
