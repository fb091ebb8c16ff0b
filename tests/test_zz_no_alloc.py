"""pg_reconstruction_noalloc: the reconstruction entry point for callers that cannot allocate
device memory (a pipeline that reserves all of its device memory up front, or a host that
gives this library a fixed budget).  It must give exactly the result of the allocating
pg_reconstruction -- and of the oracle -- call after call, while its scratch lives in one
fixed device array that keeps the previous call's contents."""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

MAX_TILES = 131040  # (1 MiB - 256 B control block) / two flag words per tile


def _setup():
    from poutre2_gb300 import _lib
    from poutre2_gb300.image import descriptor
    return _lib.load(), descriptor, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


# (shape, seed, Common_NL_SE, reconstruction type, dtype): consecutive calls of different sizes,
# connectivities, ranks and pixel types (both tile sides: 64 for 1-4 byte pixels, 32 for 8-byte),
# so each starts from whatever the previous one left in the shared scratch
CASES = [((700, 900), 1, 2, 1, np.uint8), ((333, 257), 2, 3, 0, np.uint8), ((130, 190), 3, 2, 1, np.float32),
         ((300, 260), 4, 2, 1, np.int64), ((97, 330), 5, 3, 0, np.float64), ((5000,), 6, 1, 1, np.int32),
         ((70, 90), 7, 2, 0, np.uint16)]
SE_NAMES = {1: "SESegmentX1D", 2: "SESquare2D", 3: "SECross2D"}


def test_noalloc_matches_the_allocating_entry_point_on_consecutive_calls():
    from poutre2_gb300 import synthetic
    L, descriptor, stream = _setup()
    for shape, seed, se, rtype, dt in CASES:
        if len(shape) == 1:
            mask = synthetic.smoothed_noise_u8((1, shape[0]), seed)[0].astype(np.int32)
        else:
            mask = synthetic.smoothed_noise_u8(shape, seed).astype(np.int32)
        marker = np.clip(mask - 20, 0, 255) if rtype == 1 else np.clip(mask + 20, 0, 255)
        m = torch.from_numpy(marker.astype(dt)).cuda()
        k = torch.from_numpy(mask.astype(dt)).cuda()
        out_ref = torch.empty_like(k)
        out_na = torch.full_like(k, 7)
        dm, dk, dr, dn = descriptor(m), descriptor(k), descriptor(out_ref), descriptor(out_na)
        assert L.pg_reconstruction(rtype, ctypes.byref(dm), ctypes.byref(dk), se, ctypes.byref(dr), stream) == 0
        assert L.pg_reconstruction_noalloc(rtype, ctypes.byref(dm), ctypes.byref(dk), se, ctypes.byref(dn), stream) == 0
        assert L.pg_check_device(stream) == 0
        assert torch.equal(out_ref, out_na), (shape, se, rtype, dt)
        exp = oracle.reconstruct(marker.astype(dt), mask.astype(dt), SE_NAMES[se], rtype == 1)
        np.testing.assert_array_equal(out_na.cpu().numpy(), exp, err_msg=str((shape, se, rtype, dt)))


def _shape_only(descriptor, dtype, shape):
    """Descriptors whose shapes claim `shape`, at distinct addresses 2**40 bytes apart (so that no two
    claimed buffers overlap): the entry point must reject them on the host, from the shape alone,
    before any device work -- nothing is ever read or written through these pointers."""
    ds = []
    for k in range(3):
        d = descriptor(torch.zeros((4, 4), dtype=dtype, device="cuda"))
        d.data = (k + 1) << 40
        d.rank = len(shape)
        for i, v in enumerate(shape):
            d.shape[i] = v
        ds.append(d)
    return ds


def test_noalloc_size_limit_of_its_fixed_scratch():
    L, descriptor, stream = _setup()
    # 1..4-byte pixels: 64x64 tiles; 400 x 400 tiles = 160000 > 131040
    a, b, o = _shape_only(descriptor, torch.uint8, (64 * 400, 64 * 400))
    rc = L.pg_reconstruction_noalloc(1, ctypes.byref(a), ctypes.byref(b), 2, ctypes.byref(o), stream)
    assert rc == 1 and b"fixed scratch" in L.pg_last_error()
    # 8-byte pixels: 32x32 tiles; MAX_TILES + 1 tiles is refused, MAX_TILES is the limit itself
    a, b, o = _shape_only(descriptor, torch.float64, (32 * 3, 32 * 43681))  # 131043 tiles
    rc = L.pg_reconstruction_noalloc(1, ctypes.byref(a), ctypes.byref(b), 2, ctypes.byref(o), stream)
    assert rc == 1 and b"131043 tiles" in L.pg_last_error()
    a, b, o = _shape_only(descriptor, torch.int64, (32, 32 * (MAX_TILES + 1)))
    rc = L.pg_reconstruction_noalloc(1, ctypes.byref(a), ctypes.byref(b), 2, ctypes.byref(o), stream)
    assert rc == 1 and str(MAX_TILES).encode() in L.pg_last_error()


def test_noalloc_refuses_volumes_and_keeps_the_reference_checks():
    L, descriptor, stream = _setup()
    v = torch.zeros((4, 5, 6), dtype=torch.uint8, device="cuda")
    vk, vo = v.clone(), torch.empty_like(v)  # held: a descriptor keeps only the address
    m, k, o = descriptor(v), descriptor(vk), descriptor(vo)
    assert L.pg_reconstruction_noalloc(1, ctypes.byref(m), ctypes.byref(k), 9, ctypes.byref(o), stream) == 3
    assert b"1D and 2D" in L.pg_last_error()
    x = torch.zeros((8, 8), dtype=torch.uint8, device="cuda")
    y, z = x.clone(), torch.empty_like(x)
    dx, dy, dz = descriptor(x), descriptor(y), descriptor(z)
    # output aliasing the mask: PG_ERR_ALIASING, as pg_reconstruction
    assert L.pg_reconstruction_noalloc(1, ctypes.byref(dy), ctypes.byref(dx), 2, ctypes.byref(dx), stream) == 5
    # a 3D SE on an image: PG_ERR_UNSUPPORTED_SE, as pg_reconstruction
    assert L.pg_reconstruction_noalloc(1, ctypes.byref(dy), ctypes.byref(dx), 9, ctypes.byref(dz), stream) == 3
