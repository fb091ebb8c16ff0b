"""The TMA-tiled 3x3 / 3x3x3 kernels (csrc/small_tile.cu): u8, u16, i32 and f32 images and volumes whose
rows are a multiple of 16 bytes take them for the 2D and 3D squares and crosses and the X / Y segments
(the Z segment stays on the slice-streaming kernel); the result must equal
the oracle's static-SE Erode / Dilate (ero_dil_static.cpp:229-306) bit for bit.  The shapes put the
tile's columns (64 words: 256 u8 / 128 u16 pixels), its rows (2D: 64, with a thread per 16-byte quad for
u8 and per word for wider pixels; 3D: 8), its slices (8) and
the image border in every relative position; constant images at the type's extremes check the neutral
value outside the image (the erosion's maximum replaces TMA's zero fill)."""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

SES = ["SESquare2D", "SECross2D", "SESegmentX2D", "SESegmentY2D"]
SES3 = ["SESquare3D", "SECross3D", "SESegmentX3D", "SESegmentY3D", "SESegmentZ3D"]
SHAPES = {np.uint8: [(1, 16), (2, 32), (3, 16), (63, 48), (64, 256), (65, 272), (66, 512), (127, 256),
                     (128, 512), (129, 1040), (130, 272), (257, 784)],
          np.uint16: [(1, 8), (2, 16), (3, 8), (63, 24), (64, 128), (65, 136), (66, 256), (129, 520),
                      (257, 392)]}
SHAPES3 = {np.uint8: [(1, 1, 16), (1, 3, 32), (2, 17, 48), (8, 16, 256), (9, 15, 272), (10, 18, 64),
                      (17, 33, 528), (33, 20, 80)],
           np.uint16: [(1, 1, 8), (1, 3, 16), (2, 17, 24), (8, 16, 128), (9, 15, 136), (10, 18, 32),
                       (17, 33, 264), (33, 20, 40)]}


def _op(se_name, x, out, dil, it=1):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    (llm.Dilate if dil else llm.Erode)(x, getattr(Common_NL_SE, se_name), it, out)


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("se", SES)
def test_small_tile_matches_the_oracle(dt, se):
    rng = np.random.default_rng(len(se) * 7 + np.dtype(dt).itemsize)
    for shape in SHAPES[dt]:
        a = rng.integers(0, np.iinfo(dt).max + 1, shape).astype(dt)
        x = torch.from_numpy(a).cuda()
        for dil in (True, False):
            out = torch.full_like(x, 7)
            _op(se, x, out, dil)
            np.testing.assert_array_equal(out.cpu().numpy(), oracle.erode_dilate_static(a, se, 1, dil),
                                          err_msg=f"{shape} {se} dilate={dil}")


@pytest.mark.parametrize("dt", [np.int32, np.float32])
@pytest.mark.parametrize("se", SES + SES3[:4])
def test_small_tile_wide_pixels(dt, se):
    """i32 / f32 (one pixel per word): the neutral value outside the image is the type's lowest / highest
    for both operators (TMA's zero fill is neither)."""
    rng = np.random.default_rng(len(se) + np.dtype(dt).itemsize)
    shapes = [(1, 4), (3, 12), (65, 68), (130, 132)] if se.endswith("2D") else [(1, 1, 4), (9, 17, 68), (10, 18, 8)]
    for shape in shapes:
        if dt == np.int32:
            a = rng.integers(-2**31, 2**31, shape, dtype=np.int64).astype(np.int32)
            neg = np.full(shape, -5, np.int32)
        else:
            a = rng.standard_normal(shape).astype(np.float32)
            neg = np.full(shape, -5.0, np.float32)
        for img in (a, neg, -neg):
            x = torch.from_numpy(img).cuda()
            for dil in (True, False):
                out = torch.full_like(x, 7)
                _op(se, x, out, dil)
                np.testing.assert_array_equal(out.cpu().numpy(), oracle.erode_dilate_static(img, se, 1, dil),
                                              err_msg=f"{shape} {se} dilate={dil}")


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
def test_small_tile_extremes_and_iterations(dt):
    top = np.iinfo(dt).max
    rng = np.random.default_rng(3)
    for shape in ((1, 16), (129, 272)):
        for a in (np.full(shape, top, dt), np.zeros(shape, dt),
                  rng.choice(np.array([0, top], dt), shape), rng.integers(0, 3, shape).astype(dt)):
            x = torch.from_numpy(a).cuda()
            for se in SES:
                for dil in (True, False):
                    for it in (1, 2, 3):
                        out = torch.empty_like(x)
                        _op(se, x, out, dil, it)
                        np.testing.assert_array_equal(out.cpu().numpy(), oracle.erode_dilate_static(a, se, it, dil),
                                                      err_msg=f"{shape} {se} dilate={dil} iter={it}")


def test_small_tile_large_image_status_clean():
    """4096 x 4096 u8 square: size-independent properties (the dilation is extensive and equals the
    max of the three row-shifted horizontal maxima), the oracle on a crop, and no tile wait ran out."""
    from poutre2_gb300 import _lib
    rng = np.random.default_rng(9)
    a = rng.integers(0, 256, (4096, 4096)).astype(np.uint8)
    x = torch.from_numpy(a).cuda()
    out = torch.empty_like(x)
    _op("SESquare2D", x, out, True)
    hx = x.clone()
    _op("SESegmentX2D", x, hx, True)
    hy = torch.empty_like(x)
    _op("SESegmentY2D", hx, hy, True)
    assert torch.equal(out, hy)
    o = out.cpu().numpy()
    assert (o >= a).all()
    crop = a[2000:2300, 1000:1312]
    np.testing.assert_array_equal(o[2001:2299, 1001:1311],
                                  oracle.erode_dilate_static(crop, "SESquare2D", 1, True)[1:-1, 1:-1])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _lib.load().pg_check_device(stream) == 0


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("se", SES3)
def test_small_tile_volumes_match_the_oracle(dt, se):
    rng = np.random.default_rng(len(se) * 11 + np.dtype(dt).itemsize)
    top = np.iinfo(dt).max
    for shape in SHAPES3[dt]:
        for a in (rng.integers(0, top + 1, shape).astype(dt), rng.choice(np.array([0, top], dt), shape)):
            x = torch.from_numpy(a).cuda()
            for dil in (True, False):
                out = torch.full_like(x, 7)
                _op(se, x, out, dil)
                np.testing.assert_array_equal(out.cpu().numpy(), oracle.erode_dilate_static(a, se, 1, dil),
                                              err_msg=f"{shape} {se} dilate={dil}")
    a = np.full(SHAPES3[dt][4], top, dt)
    x = torch.from_numpy(a).cuda()
    out = torch.empty_like(x)
    _op(se, x, out, False, 2)
    np.testing.assert_array_equal(out.cpu().numpy(), a)


def test_small_tile_cube_large_volume():
    """256^3 u8 cube erosion: equal to the X, Y and Z segments applied in turn (the cube is their
    product), anti-extensive, and no tile wait ran out."""
    from poutre2_gb300 import _lib
    rng = np.random.default_rng(4)
    a = rng.integers(0, 256, (256, 256, 256)).astype(np.uint8)
    x = torch.from_numpy(a).cuda()
    out = torch.empty_like(x)
    _op("SESquare3D", x, out, False)
    t1, t2 = torch.empty_like(x), torch.empty_like(x)
    _op("SESegmentX3D", x, t1, False)
    _op("SESegmentY3D", t1, t2, False)
    _op("SESegmentZ3D", t2, t1, False)
    assert torch.equal(out, t1)
    assert (out.cpu().numpy() <= a).all()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _lib.load().pg_check_device(stream) == 0
