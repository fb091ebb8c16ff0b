"""45- and 135-degree segments through the TMA parallelogram tiles (csrc/diag.cu): u16, i32 and f32
images with rows of a multiple of 16 bytes, half lengths 7, 15 and 31, against the oracle's runtime
neighbour list (ero_dil_runtime_nl_se_t.hpp:129-193, clipped at the border).  The shapes put tile
rows, tile columns and image borders in every relative position: images smaller than one tile, one row,
one 16-byte column, heights around the tile heights (112 and 120 output rows), wide and tall ones."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(1, 8), (1, 64), (5, 8), (7, 24), (33, 16), (63, 200), (111, 136), (112, 128), (113, 120),
          (119, 256), (120, 264), (121, 64), (240, 512), (345, 96), (700, 40), (64, 1024), (500, 504)]


def _rand(rng, shape, dt):
    if dt == np.float32:
        return rng.normal(0, 100, shape).astype(np.float32)
    if dt == np.int32:
        return rng.integers(-2**31, 2**31 - 1, shape, dtype=np.int64).astype(np.int32)
    return rng.integers(0, 65536, shape).astype(dt)


@pytest.mark.parametrize("dt", [np.uint16, np.int32, np.float32])
@pytest.mark.parametrize("d", [(-1, 1), (1, 1)])
@pytest.mark.parametrize("half", [7, 15, 31])
def test_diagonal_tiles_match_the_neighbour_list(dt, d, half):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import NeighborList
    rng = np.random.default_rng(half * 10 + d[0] + 5)
    offs = NeighborList.segment(d[0], d[1], half).offsets
    for shape in SHAPES:
        if (shape[1] * np.dtype(dt).itemsize) % 16:
            continue  # not a tile shape: the streaming kernels serve it (test_gpu_parity)
        a = _rand(rng, shape, dt)
        x = torch.from_numpy(a).cuda()
        for dil in (True, False):
            out = torch.full_like(x, 7)
            (llm.DilateSE if dil else llm.ErodeSE)(x, llm.se_line(d[0], d[1], half), out)
            np.testing.assert_array_equal(out.cpu().numpy(), oracle.erode_dilate_nl(a, offs, dil),
                                          err_msg=f"{shape} dilate={dil}")


def test_diagonal_tiles_opening_is_idempotent_and_status_clean():
    """Opening by the 45-degree segment twice = once (size-independent check at 2048 x 2048), and no tile
    wait ran out (pg_check_device)."""
    import ctypes
    from poutre2_gb300 import _lib, llm
    rng = np.random.default_rng(3)
    x = torch.from_numpy(rng.integers(0, 65536, (2048, 2048)).astype(np.uint16)).cuda()
    o1, o2 = torch.empty_like(x), torch.empty_like(x)
    for d in ((-1, 1), (1, 1)):
        llm.Opening(x, llm.se_line(d[0], d[1], 31), o1)
        llm.Opening(o1, llm.se_line(d[0], d[1], 31), o2)
        assert torch.equal(o1, o2)
        assert bool((o1.to(torch.int32) <= x.to(torch.int32)).all())  # anti-extensive
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _lib.load().pg_check_device(stream) == 0
