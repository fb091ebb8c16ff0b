"""Vertical, 45- and 135-degree segments through the TMA parallelogram tiles (csrc/diag.cu): u8, u16,
i32 and f32 images with rows of a multiple of 16 bytes, half lengths 7 (not u8), 15 and 31 -- the
erosion / dilation by the diagonal segments, and the opening / closing by the vertical and diagonal
segments in one pass, and the gradient by them -- against the oracle: the runtime neighbour list of the segment
(ero_dil_runtime_nl_se_t.hpp:129-193, clipped at the border) and, for the openings, the oracle's
erosion followed by its dilation.  The shapes put tile rows, tile columns and image borders in every
relative position: images smaller than one tile, one row, one 16-byte column, heights around the
tile heights (104-192 output rows), wide and tall ones."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(1, 16), (1, 64), (5, 16), (7, 32), (33, 16), (63, 208), (103, 128), (105, 136), (111, 144),
          (112, 128), (117, 120), (121, 64), (193, 96), (240, 512), (345, 96), (700, 48), (64, 1024),
          (500, 512)]
TYPES = [np.uint8, np.uint16, np.int32, np.float32]


def _rand(rng, shape, dt):
    if dt == np.float32:
        return rng.normal(0, 100, shape).astype(np.float32)
    if dt == np.int32:
        return rng.integers(-2**31, 2**31 - 1, shape, dtype=np.int64).astype(np.int32)
    return rng.integers(0, np.iinfo(dt).max + 1, shape).astype(dt)


def _tile_shapes(dt):
    return [s for s in SHAPES if (s[1] * np.dtype(dt).itemsize) % 16 == 0]


def _halves(dt):
    return [15, 31] if dt == np.uint8 else [7, 15, 31]


def _ero_dil(a, d, half, dil):
    from poutre2_gb300.se import NeighborList
    return oracle.erode_dilate_nl(a, NeighborList.segment(d[0], d[1], half).offsets, dil)


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("d", [(-1, 1), (1, 1)])
def test_diagonal_tiles_match_the_neighbour_list(dt, d):
    from poutre2_gb300 import llm
    for half in _halves(dt):
        rng = np.random.default_rng(half * 10 + d[0] + 5)
        for shape in _tile_shapes(dt):
            a = _rand(rng, shape, dt)
            x = torch.from_numpy(a).cuda()
            for dil in (True, False):
                out = torch.full_like(x, 7)
                (llm.DilateSE if dil else llm.ErodeSE)(x, llm.se_line(d[0], d[1], half), out)
                np.testing.assert_array_equal(out.cpu().numpy(), _ero_dil(a, d, half, dil),
                                              err_msg=f"{shape} half={half} dilate={dil}")


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("d", [(-1, 1), (1, 0), (1, 1)])
def test_one_pass_openings_and_closings_by_segments(dt, d):
    from poutre2_gb300 import llm
    for half in _halves(dt):
        rng = np.random.default_rng(half * 100 + d[0] * 3 + d[1] + 11)
        for shape in _tile_shapes(dt):
            a = _rand(rng, shape, dt)
            x = torch.from_numpy(a).cuda()
            e, di = _ero_dil(a, d, half, False), _ero_dil(a, d, half, True)
            for fn, exp in ((llm.Opening, _ero_dil(e, d, half, True)), (llm.Closing, _ero_dil(di, d, half, False))):
                out = torch.full_like(x, 7)
                fn(x, llm.se_line(d[0], d[1], half), out)
                np.testing.assert_array_equal(out.cpu().numpy(), exp, err_msg=f"{fn.__name__} {shape} half={half}")


def _grad(d, e):
    if d.dtype == np.int32:  # wraps like the difference kernel's int arithmetic
        return (d.view(np.uint32) - e.view(np.uint32)).view(np.int32)
    return (d - e).astype(d.dtype)


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("d", [(-1, 1), (1, 0), (1, 1)])
def test_one_pass_gradients_by_segments(dt, d):
    """Dilation - erosion by the segment from one scan of one tile; pixels of a line outside the image
    repeat the line's nearest image pixel, which leaves both clipped extrema unchanged."""
    from poutre2_gb300 import llm
    for half in _halves(dt):
        rng = np.random.default_rng(half * 7 + d[0] * 5 + d[1] + 3)
        for shape in _tile_shapes(dt):
            a = _rand(rng, shape, dt)
            x = torch.from_numpy(a).cuda()
            out = torch.full_like(x, 7)
            llm.Gradient(x, llm.se_line(d[0], d[1], half), out)
            exp = _grad(_ero_dil(a, d, half, True), _ero_dil(a, d, half, False))
            np.testing.assert_array_equal(out.cpu().numpy(), exp, err_msg=f"{shape} half={half}")


@pytest.mark.parametrize("dt", [np.uint16, np.float32])
def test_vertical_segment_forms_take_the_one_pass_opening(dt):
    """The vertical segment as a line SE, a (k, 0) rectangle and k iterations of SESegmentY2D: the same
    opening and closing."""
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(21)
    a = _rand(rng, (300, 256), dt)
    x = torch.from_numpy(a).cuda()
    for k in (7, 15, 31):
        e, di = _ero_dil(a, (1, 0), k, False), _ero_dil(a, (1, 0), k, True)
        for fn, exp in ((llm.Opening, _ero_dil(e, (1, 0), k, True)), (llm.Closing, _ero_dil(di, (1, 0), k, False))):
            for se in (llm.se_line(1, 0, k), llm.se_line(-1, 0, k), llm.se_rect(k, 0),
                       llm.se_static(Common_NL_SE.SESegmentY2D, k)):
                out = torch.full_like(x, 7)
                fn(x, se, out)
                np.testing.assert_array_equal(out.cpu().numpy(), exp, err_msg=f"{fn.__name__} k={k}")


def test_diagonal_tiles_opening_is_idempotent_and_status_clean():
    """Opening by the segments twice = once (size-independent check at 2048 x 2048), the opening is
    anti-extensive, and no tile wait ran out (pg_check_device)."""
    import ctypes
    from poutre2_gb300 import _lib, llm
    rng = np.random.default_rng(3)
    x = torch.from_numpy(rng.integers(0, 65536, (2048, 2048)).astype(np.uint16)).cuda()
    o1, o2 = torch.empty_like(x), torch.empty_like(x)
    for d in ((-1, 1), (1, 1), (1, 0)):
        llm.Opening(x, llm.se_line(d[0], d[1], 31), o1)
        llm.Opening(o1, llm.se_line(d[0], d[1], 31), o2)
        assert torch.equal(o1, o2)
        assert bool((o1.to(torch.int32) <= x.to(torch.int32)).all())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _lib.load().pg_check_device(stream) == 0
