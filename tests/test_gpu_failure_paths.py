"""Failure paths on the GPU, without a GPU fault.

poutre2 throws std::runtime_error where its reconstruction cannot finish or a temporary cannot be
allocated (include/poutre/base/config.hpp:203-214).  Here the device gives up instead of hanging: every
wait of the reconstruction kernels is bounded and its round / visit count is capped, and a give-up is
recorded in a device status word that pg_check_device returns.  The tests lower those limits through the
test hook pg_debug_set_limits so that they run out on an ordinary input (nothing else is changed: no bad
address, no trap, no endless loop), check PG_ERR_NOT_CONVERGED, and check that the next call on the same
context succeeds and is exact.  Allocation failure is injected on the host (pg_debug_fail_allocations)."""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

NOT_CONVERGED, OUT_OF_MEMORY = 9, 8


@pytest.fixture()
def L():
    from poutre2_gb300 import _lib
    lib = _lib.load()
    yield lib
    assert lib.pg_debug_set_limits(0, 0) == 0
    assert lib.pg_debug_fail_allocations(0) == 0


def serpentine(H, W, step, dt):
    """A one-pixel corridor winding through the image: reconstruction has to carry the marker's value
    along the whole corridor, visiting every tile on the path many times."""
    f = np.zeros((H, W), np.uint8)
    rows = list(range(0, H, step))
    for i, r in enumerate(rows):
        f[r, :] = 100
        if i + 1 < len(rows):
            c = W - 1 if i % 2 == 0 else 0
            f[r:rows[i + 1] + 1, c] = 100
    marker = np.zeros_like(f)
    marker[0, 0] = 100
    return marker.astype(dt), f.astype(dt)


def run(L, marker, mask, out):
    from poutre2_gb300.image import descriptor
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dm, dk, do = descriptor(marker), descriptor(mask), descriptor(out)
    assert L.pg_reconstruction(1, ctypes.byref(dm), ctypes.byref(dk), 2, ctypes.byref(do), s) == 0
    return L.pg_check_device(s)


@pytest.mark.parametrize("dt", [np.uint8, np.float32, np.int64])  # worklist kernel (<= 4 bytes), round kernel (8)
def test_visit_cap_gives_up_then_the_next_call_succeeds(L, dt):
    mk, f = serpentine(256, 256, 4, dt)
    m, k = torch.from_numpy(mk).cuda(), torch.from_numpy(f).cuda()
    out = torch.empty_like(k)
    assert L.pg_debug_set_limits(1, 0) == 0  # one round / one visit per tile on average
    assert run(L, m, k, out) == NOT_CONVERGED
    assert b"did not converge" in L.pg_last_error()
    assert L.pg_debug_set_limits(0, 0) == 0
    assert run(L, m, k, out) == 0
    np.testing.assert_array_equal(out.cpu().numpy(), oracle.reconstruct(mk, f, "SESquare2D", True))


@pytest.mark.parametrize("dt", [np.uint8, np.int64])
def test_wait_limit_runs_out_then_the_next_call_succeeds(L, dt):
    # with a 1 ns limit the first wait of any CTA (the grid barrier after the set-up phase, or an
    # empty worklist) runs out at once and the kernel returns
    mk, f = serpentine(512, 512, 4, dt)
    m, k = torch.from_numpy(mk).cuda(), torch.from_numpy(f).cuda()
    out = torch.empty_like(k)
    assert L.pg_debug_set_limits(0, 1) == 0
    assert run(L, m, k, out) == NOT_CONVERGED
    assert L.pg_debug_set_limits(0, 0) == 0
    assert run(L, m, k, out) == 0
    np.testing.assert_array_equal(out.cpu().numpy(), oracle.reconstruct(mk, f, "SESquare2D", True))
    assert L.pg_check_device(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0  # cleared


def test_injected_allocation_failure_is_out_of_memory(L):
    from poutre2_gb300 import geo
    from poutre2_gb300._lib import PoutreError
    from poutre2_gb300.se import Common_NL_SE
    f = np.random.default_rng(3).integers(0, 256, (64, 80), dtype=np.uint8)
    x = torch.from_numpy(f).cuda()
    out = torch.empty_like(x)
    assert L.pg_debug_fail_allocations(1) == 0
    with pytest.raises(PoutreError, match="OUT_OF_MEMORY"):
        geo.h_convex(x, 10, Common_NL_SE.SESquare2D, out)  # needs one temporary
    geo.h_convex(x, 10, Common_NL_SE.SESquare2D, out)  # the failure was used up
    np.testing.assert_array_equal(out.cpu().numpy(), oracle.h_convex(f, 10, "SESquare2D"))


def test_hooks_need_no_gpu_state_beyond_the_limits(L):
    assert L.pg_debug_set_limits(-1, 0) == 1
    assert L.pg_debug_fail_allocations(-1) == 1
