"""pg_reconstruction_noalloc: the reconstruction entry point for callers that cannot allocate
device memory (a pipeline that reserves all of its device memory up front, or a host that
gives this library a fixed budget).  It must give exactly the result of the allocating
pg_reconstruction, call after call, while its scratch lives in one fixed device array that
keeps the previous call's contents."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup():
    from poutre2_gb300 import _lib
    from poutre2_gb300.image import descriptor
    return _lib.load(), descriptor, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_the_allocating_entry_point_on_consecutive_calls():
    from poutre2_gb300 import synthetic
    L, descriptor, stream = _setup()
    # two calls in a row: different sizes, connectivities and types, so the second starts
    # from whatever the first left in the shared scratch
    cases = [((700, 900), 1, 2, 1, np.uint8), ((333, 257), 2, 3, 0, np.uint8), ((130, 190), 3, 2, 1, np.float32)]
    for shape, seed, se, rtype, dt in cases:
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


def test_noalloc_rejects_images_beyond_its_fixed_scratch():
    L, descriptor, stream = _setup()
    x = torch.zeros((4, 4), dtype=torch.uint8, device="cuda")
    big = descriptor(x)
    big.shape[0] = 64 * 400
    big.shape[1] = 64 * 400  # 160000 tiles > 131040; rejected on the host before any device work
    big2 = descriptor(torch.zeros((4, 4), dtype=torch.uint8, device="cuda"))
    big2.shape[0], big2.shape[1] = big.shape[0], big.shape[1]
    out = descriptor(torch.zeros((4, 4), dtype=torch.uint8, device="cuda"))
    out.shape[0], out.shape[1] = big.shape[0], big.shape[1]
    rc = L.pg_reconstruction_noalloc(1, ctypes.byref(big), ctypes.byref(big2), 2, ctypes.byref(out), stream)
    assert rc == 1 and b"fixed scratch" in L.pg_last_error()
