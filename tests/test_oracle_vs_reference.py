"""Cross-check the C restatement (oracle) against poutre2's own implementation
(oracle/_ref, compiled from the reference sources) on seeded random inputs.

Skipped when oracle/_ref was not built (the reference tree is neither mounted nor staged)."""
import numpy as np
import pytest

import oracle
from oracle import ref

pytestmark = pytest.mark.skipif(not ref.available(), reason="oracle/_ref/libpoutre_ref.so not built")

REF_TYPES = [np.uint8, np.int32, np.int64, np.float32, np.float64]
SES_2D = ["SESquare2D", "SECross2D", "SESegmentX2D", "SESegmentY2D"]
SES_3D = ["SESquare3D", "SECross3D", "SESegmentX3D", "SESegmentY3D", "SESegmentZ3D"]


def rand(rng, shape, dt):
    dt = np.dtype(dt)
    if dt.kind == "f":
        return rng.standard_normal(shape).astype(dt)
    if dt == np.uint8:
        return rng.integers(0, 256, shape, dtype=np.int64).astype(dt)
    return rng.integers(-1000, 1000, shape, dtype=np.int64).astype(dt)


def smooth_u8(rng, shape, sigma=2.0):
    from scipy.ndimage import gaussian_filter
    x = gaussian_filter(rng.random(shape), sigma)
    x = (x - x.min()) / max(x.max() - x.min(), 1e-12)
    return np.rint(x * 255).astype(np.uint8)


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("se", SES_2D)
@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (7, 1), (13, 17), (64, 33)])
def test_static_2d(dt, se, shape):
    rng = np.random.default_rng(hash((str(dt), se, shape)) % 2**32)
    a = rand(rng, shape, dt)
    for dil in (True, False):
        for it in (1, 2, 3):
            np.testing.assert_array_equal(oracle.erode_dilate_static(a, se, it, dil),
                                          ref.erode_dilate_static(a, se, it, dil))


@pytest.mark.parametrize("se", SES_3D)
@pytest.mark.parametrize("shape", [(5, 5, 5), (4, 6, 7), (3, 1, 8)])
def test_static_3d_matches_reference_neighbor_list(se, shape):
    from poutre2_gb300.se import predefined_offsets
    rng = np.random.default_rng(sum(shape))
    a = rand(rng, shape, np.int32)
    for dil in (True, False):
        np.testing.assert_array_equal(oracle.erode_dilate_static(a, se, 1, dil),
                                      ref.erode_dilate_nl(a, predefined_offsets(se), dil))


@pytest.mark.parametrize("se", ["SESquare3D", "SECross3D"])
def test_reference_static_3d_defect_is_confined_to_slice_path(se):
    """The reference's slice-wise SESquare3D/SECross3D specialisation loses track of its
    slice buffers (ero_dil_static_se_t.hpp:761-915): it disagrees with its own
    neighbour-list path on random volumes, and agrees on a 3x3x3 cube of equal slices (the
    regime of its own known-answer test)."""
    from poutre2_gb300.se import predefined_offsets
    rng = np.random.default_rng(1)
    a = rand(rng, (5, 5, 5), np.int32)
    assert not np.array_equal(ref.erode_dilate_static(a, se, 1, True), ref.erode_dilate_nl(a, predefined_offsets(se), True))
    flat = np.repeat(rand(rng, (1, 3, 3), np.int32), 3, axis=0)
    np.testing.assert_array_equal(ref.erode_dilate_static(flat, se, 1, True), oracle.erode_dilate_static(flat, se, 1, True))


@pytest.mark.parametrize("dt", REF_TYPES)
def test_neighbor_list_45deg_and_5x5(dt):
    from poutre2_gb300.se import NeighborList
    rng = np.random.default_rng(7)
    a = rand(rng, (40, 37), dt)
    for nl in (NeighborList.segment(-1, 1, 6), NeighborList.rectangle(2, 2), NeighborList.segment(0, 1, 4)):
        for dil in (True, False):
            np.testing.assert_array_equal(oracle.erode_dilate_nl(a, nl.offsets, dil), ref.erode_dilate_nl(a, nl.offsets, dil))


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("half", [0, 1, 3, 15])
def test_lines(dt, half):
    rng = np.random.default_rng(half)
    a = rand(rng, (33, 33), dt)
    for axis in ("x", "y"):
        for dil in (True, False):
            np.testing.assert_array_equal(oracle.line(a, half, axis, dil), ref.line(a, half, axis, dil))
    b = rand(rng, (9, 70), dt)
    np.testing.assert_array_equal(oracle.line(b, half, "x", True), ref.line(b, half, "x", True))


def test_square_iterated_equals_rectangle():
    # 31x31 square = 3x3 square iterated 15 times = DilateY(DilateX(., 15), 15)
    rng = np.random.default_rng(3)
    a = rand(rng, (80, 80), np.float32)
    np.testing.assert_array_equal(ref.erode_dilate_static(a, "SESquare2D", 15, True), oracle.rect(a, 15, 15, True))
    np.testing.assert_array_equal(ref.erode_dilate_static(a, "SESquare2D", 15, False), oracle.rect(a, 15, 15, False))


@pytest.mark.parametrize("dt", [np.uint8, np.int32, np.int64])
@pytest.mark.parametrize("se", ["SESquare2D", "SECross2D"])
def test_reconstruction(dt, se):
    rng = np.random.default_rng(11)
    for shape in [(1, 1), (1, 30), (30, 1), (50, 61)]:
        mask = smooth_u8(rng, shape).astype(dt)
        marker = oracle.sat_sub_const(mask, 20) if dt == np.uint8 else (mask - 20).astype(dt)
        for dil in (True, False):
            mk = marker if dil else (mask + 20).astype(dt)
            np.testing.assert_array_equal(oracle.reconstruct(mk, mask, se, dil), ref.reconstruct(mk, mask, se, dil))


@pytest.mark.parametrize("kind", ["h_minima", "h_maxima", "h_concave", "h_convex",
                                  "dynamic_pseudo_opening", "dynamic_pseudo_closing"])
def test_extrema(kind):
    rng = np.random.default_rng(5)
    f = smooth_u8(rng, (60, 47))
    np.testing.assert_array_equal(getattr(oracle, kind)(f, 10, "SESquare2D"), ref.extrema(kind, f, 10, "SESquare2D"))
    g = f.astype(np.int32) * 3 - 100
    np.testing.assert_array_equal(getattr(oracle, kind)(g, 25, "SECross2D"), ref.extrema(kind, g, 25, "SECross2D"))


def test_h_maxima_binary():
    rng = np.random.default_rng(9)
    f = smooth_u8(rng, (70, 90), 3.0)
    np.testing.assert_array_equal(oracle.h_maxima_binary(f, 20), ref.h_maxima_binary(f, 20))


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("kind", ["low_leveling", "high_leveling", "leveling"])
def test_leveling(dt, kind):
    rng = np.random.default_rng(13)
    r = smooth_u8(rng, (45, 52)).astype(dt)
    m = smooth_u8(rng, (45, 52), 6.0).astype(dt)
    np.testing.assert_array_equal(getattr(oracle, kind)(r, m, "SESquare2D"), ref.leveling(kind, r, m, "SESquare2D"))


def test_uint16_composition_rule():
    # u16 has no reference PType: widen to i32, run the reference, narrow.
    rng = np.random.default_rng(21)
    a = rng.integers(0, 65536, (31, 29)).astype(np.uint16)
    for se in ("SESquare2D", "SECross2D"):
        got = oracle.erode_dilate_static(a, se, 2, True)
        exp = ref.erode_dilate_static(a.astype(np.int32), se, 2, True).astype(np.uint16)
        np.testing.assert_array_equal(got, exp)
    b = a[:29, :29].copy()  # DilateY/ErodeY need a square image
    np.testing.assert_array_equal(oracle.line(b, 5, "y", False), ref.line(b.astype(np.int32), 5, "y", False).astype(np.uint16))


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("se,rank", [("SESquare2D", 2), ("SECross2D", 2), ("SESegmentX2D", 2), ("SESegmentY2D", 2),
                                     ("SESegmentX1D", 1), ("SECross3D", 3), ("SESegmentZ3D", 3)])
@pytest.mark.parametrize("flat", [False, True])
def test_labelling(dt, se, rank, flat):
    # label_binary with negative and zero pixels (a negative pixel is foreground but joins no later
    # pixel), and label_flat_zones over a few grey levels
    rng = np.random.default_rng(hash((str(dt), se, flat)) % 2**32)
    for shape in ([(1,), (37,), (200,)] if rank == 1 else [(1, 1), (9, 13), (64, 41)] if rank == 2
                  else [(1, 1, 1), (5, 6, 7), (9, 12, 11)])[: 3]:
        shape = shape[:rank]
        if flat:
            a = rng.integers(0, 3, shape).astype(dt)
        else:
            fg = rng.random(shape) < 0.45
            vals = rng.integers(-2 if np.dtype(dt).kind in "if" else 1, 5, shape)
            a = (fg * vals).astype(dt)
        try:
            got, n = oracle.label(a, se, flat)
        except oracle.OracleError:
            continue  # float background in (0, 1e-10]: undefined in the reference
        exp, m = ref.label(a, se, flat)
        assert n == m
        np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("se,rank", [("SESquare2D", 2), ("SECross2D", 2)])
@pytest.mark.parametrize("maxima", [False, True])
def test_label_extrema(dt, se, rank, maxima):
    # label_minima / label_maxima: regional extrema of plateau-rich images (few grey levels).  The
    # reference rejects 1D images here (ArithSaturatedSubConstant has no 1D case, arith.cpp:533).
    if np.dtype(dt).kind == "f":
        pytest.skip("float regional extrema label the h-convex residue with an undefined background")
    rng = np.random.default_rng(hash((str(dt), se, maxima)) % 2**32)
    for shape in [(1, 1), (11, 14), (60, 47)]:
        a = rng.integers(0, 6, shape).astype(dt)
        got, n = oracle.label_extrema(a, se, maxima)
        exp = ref.label_extrema(a, se, maxima)
        assert n == int(exp.max())
        np.testing.assert_array_equal(got, exp)


# ----------------------------------------------------------------------------- pixel processing
def _full_range(rng, dt, shape):
    """Values over the whole range of the type, its extremes included."""
    dt = np.dtype(dt)
    if dt.kind in "iu":
        info = np.iinfo(dt)
        a = rng.integers(info.min, info.max, shape, dtype=dt, endpoint=True)
        flat = a.reshape(-1)
        flat[: 4] = [info.min, info.max, info.min, info.max][: flat.size]
        return a
    return (rng.standard_normal(shape) * 1e3).astype(dt)


# pixel counts that are multiples of 32, so that every pixel takes the reference's vector body
PIXEL_SHAPES = [(8, 16), (3, 4, 32), (32, 45)]


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("kind", ["invert", "sup", "inf", "sat_add", "sat_sub"])
def test_pixel_arith(dt, kind):
    rng = np.random.default_rng(hash((str(dt), kind)) % 2**32)
    fn = {"invert": lambda a, b: oracle.invert_image(a), "sup": oracle.sup_image, "inf": oracle.inf_image,
          "sat_add": oracle.sat_add_image, "sat_sub": oracle.sat_sub_image}[kind]
    for shape in PIXEL_SHAPES:
        a, b = _full_range(rng, dt, shape), _full_range(rng, dt, shape)
        b.reshape(-1)[:4] = b.reshape(-1)[[1, 0, 0, 1]]  # (min, max), (max, min), (min, min), (max, max)
        np.testing.assert_array_equal(fn(a, b), ref.arith(kind, a, b), err_msg=f"{kind} {shape}")


@pytest.mark.parametrize("dt_in", REF_TYPES)
@pytest.mark.parametrize("dt_out", [np.uint8, np.int64, np.float32])
@pytest.mark.parametrize("form", ["sss", "ssi", "sis", "sii", "iss", "isi", "iis", "iii"])
def test_compare_all_overloads(dt_in, dt_out, form):
    rng = np.random.default_rng(hash((str(dt_in), str(dt_out), form)) % 2**32)
    shape = (9, 13)
    a = rng.integers(0, 5, shape).astype(dt_in)
    opnds = []
    for kind, dt in zip(form, (dt_in, dt_out, dt_out)):
        opnds.append(rng.integers(0, 5, shape).astype(dt) if kind == "i" else int(rng.integers(0, 5)))
    for op in ("equal", "diff", "sup", "sup_equal", "inf", "inf_equal"):
        got = oracle.compare(a, op, *opnds, dt_out)
        exp = ref.compare(a, op, *opnds, dt_out)
        np.testing.assert_array_equal(got, exp, err_msg=f"{op} {form}")


@pytest.mark.parametrize("dt_in", REF_TYPES)
@pytest.mark.parametrize("dt_out", REF_TYPES)
def test_convert(dt_in, dt_out):
    # values every output type holds (static_cast of an out-of-range float is undefined)
    rng = np.random.default_rng(hash((str(dt_in), str(dt_out))) % 2**32)
    lo = 0 if np.dtype(dt_out) == np.uint8 or np.dtype(dt_in) == np.uint8 else -1000
    hi = 255 if np.dtype(dt_out) == np.uint8 or np.dtype(dt_in) == np.uint8 else 1000
    a = rng.uniform(lo, hi, (7, 11)).astype(dt_in)
    np.testing.assert_array_equal(oracle.convert(a, dt_out), ref.convert(a, dt_out))
    if np.dtype(dt_in).kind == "i" and np.dtype(dt_out).kind in "iu" and np.dtype(dt_out).itemsize < np.dtype(dt_in).itemsize:
        w = _full_range(rng, dt_in, (6, 8))  # modular narrowing
        np.testing.assert_array_equal(oracle.convert(w, dt_out), ref.convert(w, dt_out))


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("dilate", [True, False])
def test_compound_octagon(dt, dilate):
    rng = np.random.default_rng(hash((str(dt), dilate, "octagon")) % 2**32)
    for shape in [(1, 1), (7, 30), (41, 37)]:
        a = rand(rng, shape, dt)
        for size in range(0, 13):
            got = oracle.erode_dilate_compound(a, "Octagon", size, dilate)
            exp = ref.erode_dilate_compound(a, "Octagon", size, dilate)
            np.testing.assert_array_equal(got, exp, err_msg=f"{shape} size={size}")


@pytest.mark.parametrize("dilate", [True, False])
def test_compound_rhombicuboctahedron(dilate):
    rng = np.random.default_rng(17 + dilate)
    a = rand(rng, (9, 9, 9), np.int32)  # a cube: the reference's slice-wise 3D passes read it as such
    for size in (0, 2, 3, 4):
        got = oracle.erode_dilate_compound(a, "Rhombicuboctahedron", size, dilate)
        exp = ref.erode_dilate_compound(a, "Rhombicuboctahedron", size, dilate)
        if size >= 2:
            continue  # the reference's slice-wise SESquare3D / SECross3D passes are defective (recorded)
        np.testing.assert_array_equal(got, exp, err_msg=f"size={size}")


@pytest.mark.parametrize("dt", REF_TYPES)
@pytest.mark.parametrize("se", ["SECross3D", "SESquare3D"])
def test_geodesy_3d(dt, se):
    # reconstruction, h-extrema and leveling of volumes (the oracle is also the GPU's checker here)
    if np.dtype(dt).kind == "f":
        pytest.skip("the reference reconstructs u8, i32 and i64 only")
    rng = np.random.default_rng(hash((str(dt), se, "3d")) % 2**32)
    for shape in [(1, 1, 1), (4, 5, 6), (9, 8, 10)]:
        mask = rng.integers(0, 60, shape).astype(dt)
        for dil in (True, False):
            mk = (mask // 2).astype(dt) if dil else (mask + 25).astype(dt)
            np.testing.assert_array_equal(oracle.reconstruct(mk, mask, se, dil), ref.reconstruct(mk, mask, se, dil))
        for kind in ("h_maxima", "h_minima"):
            np.testing.assert_array_equal(getattr(oracle, kind)(mask, 7, se), ref.extrema(kind, mask, 7, se))
        marker = rng.integers(0, 60, shape).astype(dt)
        for kind in ("low_leveling", "high_leveling", "leveling"):
            np.testing.assert_array_equal(getattr(oracle, kind)(mask, marker, se), ref.leveling(kind, mask, marker, se))


@pytest.mark.parametrize("maxima", [False, True])
def test_label_extrema_3d(maxima):
    rng = np.random.default_rng(61 + maxima)
    for shape in [(1, 1, 1), (4, 5, 6), (7, 9, 8)]:
        a = rng.integers(0, 6, shape).astype(np.uint8)
        got, n = oracle.label_extrema(a, "SECross3D", maxima)
        exp = ref.label_extrema(a, "SECross3D", maxima)
        assert n == int(exp.max())
        np.testing.assert_array_equal(got, exp, err_msg=f"{shape}")


@pytest.mark.parametrize("kind", ["h_convex", "h_concave", "dynamic_pseudo_opening", "dynamic_pseudo_closing"])
def test_extrema_3d(kind):
    rng = np.random.default_rng(hash((kind, "3d")) % 2**32)
    for dt in (np.uint8, np.int32):
        for shape in [(1, 1, 1), (5, 6, 7), (8, 9, 10)]:
            f = rng.integers(0, 60, shape).astype(dt)
            np.testing.assert_array_equal(getattr(oracle, kind)(f, 7, "SECross3D"), ref.extrema(kind, f, 7, "SECross3D"),
                                          err_msg=f"{dt} {shape}")
