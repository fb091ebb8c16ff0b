"""CPU-side checks of the boundary: the C-ABI library builds for sm_103a, loads without a GPU
and exports exactly the entry points include/poutre_gb300.h declares; host-side helpers."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "poutre_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^PG_API\s+[^;(]*?\b(pg_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from poutre2_gb300 import build
    return build.build()


def test_header_declares_the_boundary():
    syms = declared_symbols()
    from poutre2_gb300._lib import EXPORTED
    assert syms == sorted(EXPORTED)
    assert len(syms) >= 30


def test_library_loads_and_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    for s in declared_symbols():
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = sorted(l.split()[-1] for l in out.splitlines() if l.split()[-1].startswith("pg_"))
    assert exported == declared_symbols()


def test_library_is_built_for_sm_103a(lib_path):
    from poutre2_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)


def test_python_binding_loads_without_gpu(lib_path):
    from poutre2_gb300 import _lib
    L = _lib.load()
    assert b"sm_103a" in L.pg_version()


def test_descriptor_rejects_cpu_tensors():
    import torch
    from poutre2_gb300._lib import PoutreError
    from poutre2_gb300.image import descriptor
    with pytest.raises(PoutreError):
        descriptor(torch.zeros(4, 4, dtype=torch.uint8))


def test_image_string_round_trip_host():
    from poutre2_gb300.image import ImageFromString, ImageToString
    s = "Scalar GINT64 2 2 3 1 -2 3 4 5 6"
    t = ImageFromString(s, device="cpu")
    assert t.shape == (2, 3) and ImageToString(t) == s
    # trailing tokens are ignored, as poutre::ImageFromString does
    assert ImageToString(ImageFromString("Scalar GUINT8 1 3 1 2 3 9 9", device="cpu")) == "Scalar GUINT8 1 3 1 2 3"


def test_structuring_elements():
    from poutre2_gb300.se import NeighborList, predefined_offsets
    assert len(predefined_offsets("SESquare3D")) == 27 and predefined_offsets("SESquare2D")[0] == (0, 0)
    seg = NeighborList.segment(-1, 1, 31)
    assert len(seg) == 63 and (-31, 31) in seg.offsets and (31, -31) in seg.offsets
    lo, hi = NeighborList.rectangle(2, 3).maximum_extension()
    assert lo == (-2, -3) and hi == (2, 3)
    assert NeighborList([(1, 2)]).Transpose().offsets == [(-1, -2)]


def test_synthetic_inputs_are_deterministic():
    from poutre2_gb300 import synthetic
    a = synthetic.smoothed_noise_u8((64, 80), 1)
    b = synthetic.smoothed_noise_u8((64, 80), 1)
    assert np.array_equal(a, b) and a.min() == 0 and a.max() == 255
    sizes = synthetic.ragged_sizes(512)
    assert len(sizes) == 512 and all(64 <= h <= 1024 and 64 <= w <= 1024 for h, w in sizes)


def test_labelling_argument_checks_need_no_gpu(lib_path):
    # the C ABI rejects, before any device work, what the reference rejects: an output that is not
    # INT64, an SE of another rank, SESquare3D (not on the GPU path), a float image for label_binary
    import ctypes
    from poutre2_gb300 import _lib
    L = _lib.load()

    def img(ptype, shape):
        d = _lib.PgImage()
        d.data, d.ptype, d.rank = 0x1000, ptype, len(shape)
        for i, s in enumerate(shape):
            d.shape[i] = s
        return d

    n = ctypes.c_int64(0)
    a, o = img(4, (8, 8)), img(32, (8, 8))
    o.data = 0x100000
    assert L.pg_label_binary(ctypes.byref(a), 2, ctypes.byref(img(4, (8, 8))), ctypes.byref(n), None) == 4  # u8 out
    assert L.pg_label_binary(ctypes.byref(a), 9, ctypes.byref(o), ctypes.byref(n), None) == 3  # 3D SE, 2D image
    a3, o3 = img(4, (4, 4, 4)), img(32, (4, 4, 4))
    o3.data = 0x100000
    assert L.pg_label_binary(ctypes.byref(a3), 10, ctypes.byref(o3), ctypes.byref(n), None) == 3  # SESquare3D
    af = img(16, (8, 8))
    assert L.pg_label_binary(ctypes.byref(af), 2, ctypes.byref(o), ctypes.byref(n), None) == 2  # float binary
    assert L.pg_label_flat_zones(ctypes.byref(a), 2, ctypes.byref(img(32, (8, 9))), ctypes.byref(n), None) == 4
    o8 = img(4, (8, 8))
    o8.data = 0x100000
    for fn in (L.pg_label_minima, L.pg_label_maxima):
        assert fn(ctypes.byref(a), 2, ctypes.byref(o8), ctypes.byref(n), None) == 4  # u8 out
        assert fn(ctypes.byref(a), 2, ctypes.byref(a), ctypes.byref(n), None) == 5  # in place
        assert fn(ctypes.byref(a), 9, ctypes.byref(o), ctypes.byref(n), None) == 3  # 3D SE, 2D image
        assert fn(ctypes.byref(af), 2, ctypes.byref(o), ctypes.byref(n), None) == 2  # float image


def test_pixel_processing_argument_checks_need_no_gpu(lib_path):
    # types, sizes, partial overlaps, CompOpType values and scalar ranges are rejected before any
    # device work, as the reference's asserts and std::get<pType> would
    import ctypes
    from poutre2_gb300 import _lib
    L = _lib.load()

    def img(ptype, shape, data):
        d = _lib.PgImage()
        d.data, d.ptype, d.rank = data, ptype, len(shape)
        for i, s in enumerate(shape):
            d.shape[i] = s
        return d

    a, b = img(8, (8, 8), 0x10000), img(8, (8, 8), 0x20000)
    o = img(8, (8, 8), 0x30000)
    wide = img(32, (8, 8), 0x30000)
    B = ctypes.byref
    assert L.pg_arith_sup_image(B(a), B(img(32, (8, 8), 0x20000)), B(o), None) == 4   # types differ
    assert L.pg_sat_add_image(B(a), B(img(8, (8, 9), 0x20000)), B(o), None) == 4      # sizes differ
    assert L.pg_arith_inf_image(B(a), B(b), B(img(8, (8, 8), 0x10000 + 12)), None) == 5  # partial overlap
    assert L.pg_arith_invert_image(B(a), B(img(8, (8, 8), 0x10004)), None) == 5
    assert L.pg_convert_into(B(a), B(img(16, (8, 8), 0x10000)), None) == 5            # must be different
    assert L.pg_copy_into(B(a), B(wide), None) == 4
    member = {4: "u8", 8: "i32", 16: "f32", 32: "i64"}

    def s(pt, v):
        sc = _lib.PgScalar()
        sc.ptype = pt
        setattr(sc.v, member[pt], v)
        return _lib.PgOperand(None, sc)
    i = lambda d: _lib.PgOperand(ctypes.pointer(d), _lib.PgScalar())  # noqa: E731
    assert L.pg_compare_image(B(a), 3, B(s(8, 1)), B(s(8, 1)), B(s(8, 0)), B(o), None) == 1     # not a CompOpType
    # a scalar that does not hold the pixel type std::get<T> asks for: PG_ERR_SCALAR_TYPE
    assert L.pg_compare_image(B(a), 4, B(s(16, 0.5)), B(s(8, 1)), B(s(8, 0)), B(o), None) == 10  # FLOAT vs INT32 input
    assert L.pg_compare_image(B(a), 4, B(s(8, 1)), B(s(8, 255)), B(s(4, 0)),
                              B(img(4, (8, 8), 0x30000)), None) == 10                        # INT32 vs UINT8 output
    assert b"unable to extract suitable type" in L.pg_last_error()
    assert L.pg_compare_image(B(a), 4, B(i(img(32, (8, 8), 0x20000))), B(s(8, 1)), B(s(8, 0)), B(o), None) == 4
    assert L.pg_compare_image(B(a), 4, B(s(8, 1)), B(i(img(8, (8, 8), 0x20000))), B(s(32, 0)), B(wide), None) == 4
    assert L.pg_compare_image(B(a), 4, B(s(8, 1)), B(s(8, 1)), B(s(8, 0)), B(img(8, (4, 16), 0x30000)), None) == 4


# pypoutre's function and enum names (python/*/*.cpp of poutre2), all present in the mirror
PYPOUTRE_NAMES = [
    "PType", "CType", "Comp", "Image", "as_sizes_compatible", "as_types_compatible", "are_images_different",
    "factory_image", "from_string", "to_string", "arith_invert_image", "arith_inf_image", "arith_sup_image",
    "arith_saturated_add_image", "arith_saturated_sub_image", "arith_saturated_add_constant",
    "arith_saturated_sub_constant", "compare", "clone", "clone_geometry", "convert", "convert_geometry",
    "copy_into", "convert_into", "se_type", "static_nl_se", "static_compound_se", "erode", "dilate", "dilateX",
    "dilateY", "erodeX", "erodeY", "RecType", "h_minima", "h_maxima", "h_concave", "h_convex",
    "dynamic_pseudo_closing", "dynamic_pseudo_opening", "high_leveling", "low_leveling", "leveling",
    "label_binary", "label_flat_zones", "label_maxima", "label_minima"]


def test_pypoutre_mirror_names_and_enums():
    from poutre2_gb300 import pypoutre as pp
    for name in PYPOUTRE_NAMES:
        assert hasattr(pp, name), name
    assert [m.name for m in pp.static_nl_se] == ["segx1d", "square2d", "cross2d", "segx2d", "segy2d", "segx3d",
                                                 "segy3d", "segz3d", "cross3d", "square3d"]
    assert {m.name for m in pp.Comp} == {"Diff", "Equal", "Inf", "Sup", "InfEqual", "SupEqual"}
    assert int(pp.Comp.Sup) == 4 and int(pp.PType.GrayUINT8) == 4 and int(pp.RecType.dilate) == 1
    with pytest.raises(Exception):
        pp.Image(__import__("torch").zeros(3, 3))  # a host tensor is no device image


def test_pixel_and_pypoutre_refuse_host_images():
    # no CPU path: host tensors are refused before the library is called
    import torch
    from poutre2_gb300 import pixel
    from poutre2_gb300 import pypoutre as pp
    from poutre2_gb300._lib import PoutreError
    h = torch.zeros(4, 4, dtype=torch.uint8)
    with pytest.raises(PoutreError):
        pixel.ArithSupImage(h, h, torch.zeros_like(h))
    with pytest.raises(PoutreError):
        pixel.CompareImage(h, pixel.CompOpType.CompOpSup, 1, 255, 0, torch.zeros_like(h))
    with pytest.raises(PoutreError):
        pp.dilate(h, pp.static_nl_se.square2d, 1, torch.zeros_like(h))
    with pytest.raises(PoutreError):
        pp.label_maxima(h, pp.static_nl_se.square2d, torch.zeros(4, 4, dtype=torch.int64))


def test_square3d_reconstruction_is_refused_before_device_work(lib_path):
    # poutre2's SESquare3D reconstruction stops short of the fixpoint on thin volumes: not on the GPU path
    import ctypes
    from poutre2_gb300 import _lib
    L = _lib.load()

    def img(shape, data):
        d = _lib.PgImage()
        d.data, d.ptype, d.rank = data, 4, len(shape)
        for i, s in enumerate(shape):
            d.shape[i] = s
        return d

    m, k, o = img((4, 4, 4), 0x10000), img((4, 4, 4), 0x20000), img((4, 4, 4), 0x30000)
    B = ctypes.byref
    assert L.pg_reconstruction(1, B(m), B(k), 10, B(o), None) == 3
    h = _lib.scalar(4, 5)
    assert L.pg_h_maxima(B(m), B(h), 10, B(o), None) == 3


def test_exact_scalars_cross_the_boundary_without_rounding():
    """pg_scalar carries every int64 value exactly (a double would round 2**62 + 1) and a Python value
    that the pixel type cannot hold is refused like poutre2's std::get<T> refuses the variant."""
    import numpy as np
    from poutre2_gb300 import _lib
    v = 2**62 + 1
    assert _lib.scalar(32, v).v.i64 == v and _lib.scalar(32, v).ptype == 32
    assert _lib.scalar(32, -2**63).v.i64 == -2**63
    assert _lib.scalar(4, 20.0).v.u8 == 20
    assert _lib.scalar(16, 0.1).v.f32 == np.float32(0.1)
    assert _lib.scalar(8, np.float64(1.5)).ptype == 64  # a numpy scalar keeps its own type
    for pt, bad in ((4, 256), (4, -1), (8, 0.5), (32, 2**63), (128, 70000), (16, "x"), (8, True)):
        try:
            _lib.scalar(pt, bad)
        except _lib.PoutreError as e:
            assert e.status == 10
        else:
            raise AssertionError((pt, bad))
