"""The octagon's passes in one shared-memory tile kernel (csrc/octagon.cu): u8 and u16 images with rows
of a multiple of 16 bytes, sizes 2..16 (the tile from 5 passes for u8, from 3 for u16; fewer take the
separate passes), dilation and erosion, against the oracle's compound
Erode / Dilate (ero_dil_compound_static_se_t.hpp:34-160, pinned against poutre2's compound path).
The shapes put tile columns (56 / 48 words), tile rows (128 - 2n) and the image border in every
relative position: one row, one 16-byte column, images smaller than a tile, several tiles across and
down."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

SHAPES = {np.uint8: [(1, 16), (3, 32), (17, 48), (96, 224), (110, 240), (127, 400), (300, 512), (513, 1008)],
          np.uint16: [(1, 8), (3, 16), (17, 24), (96, 112), (110, 120), (127, 200), (300, 256), (513, 520)]}


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
@pytest.mark.parametrize("size", [2, 3, 4, 5, 8, 9, 12, 16])
def test_octagon_tile_matches_the_compound_passes(dt, size):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Compound_NL_SE
    rng = np.random.default_rng(size * 31 + np.dtype(dt).itemsize)
    for shape in SHAPES[dt]:
        a = rng.integers(0, np.iinfo(dt).max + 1, shape).astype(dt)
        x = torch.from_numpy(a).cuda()
        for dil in (True, False):
            out = torch.full_like(x, 7)
            (llm.Dilate if dil else llm.Erode)(x, Compound_NL_SE.Octagon, size, out)
            np.testing.assert_array_equal(out.cpu().numpy(), oracle.erode_dilate_compound(a, "Octagon", size, dil),
                                          err_msg=f"{shape} size={size} dilate={dil}")


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
def test_iterated_cross_takes_the_tile_kernel(dt):
    """Erode / Dilate by SECross2D iterated 2..16 times (the diamond) in one tile launch, against the
    oracle's iterated passes (ero_dil_static.cpp:229-306)."""
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(77 + np.dtype(dt).itemsize)
    for shape in SHAPES[dt]:
        a = rng.integers(0, np.iinfo(dt).max + 1, shape).astype(dt)
        x = torch.from_numpy(a).cuda()
        for it in (2, 3, 5, 7, 16):
            for dil in (True, False):
                out = torch.full_like(x, 7)
                (llm.Dilate if dil else llm.Erode)(x, Common_NL_SE.SECross2D, it, out)
                np.testing.assert_array_equal(out.cpu().numpy(), oracle.erode_dilate_static(a, "SECross2D", it, dil),
                                              err_msg=f"{shape} iter={it} dilate={dil}")


def test_octagon_tile_large_image_status_clean():
    """4096 x 4096 u8, size 10: the octagon is the dilation by itself only up to the border, so check
    the size-independent properties: extensive, idempotent under max with the input, equal to the
    oracle on a central crop far from the border, and no tile wait ran out."""
    import ctypes
    from poutre2_gb300 import _lib, llm
    from poutre2_gb300.se import Compound_NL_SE
    rng = np.random.default_rng(5)
    a = rng.integers(0, 256, (4096, 4096)).astype(np.uint8)
    x = torch.from_numpy(a).cuda()
    out = torch.empty_like(x)
    llm.Dilate(x, Compound_NL_SE.Octagon, 10, out)
    o = out.cpu().numpy()
    assert (o >= a).all()
    crop = a[1000:1300, 2000:2304]
    exp = oracle.erode_dilate_compound(crop, "Octagon", 10, True)
    np.testing.assert_array_equal(o[1010:1290, 2010:2294], exp[10:-10, 10:-10])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _lib.load().pg_check_device(stream) == 0
