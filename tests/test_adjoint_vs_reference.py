"""The flat-morphology adjoint's oracle pinned to poutre2 itself (CPU).

1. The oracle's forward (`or_flat2d_forward`) equals poutre2's own float32
   Dilate/Erode(SESquare2D, iter=r) (src/low_level_morpho/ero_dil_static.cpp:229-306) and its runtime
   (2r+1)^2 neighbour list (include/poutre/low_level_morpho/details/ero_dil_runtime_nl_se_t.hpp:129-193),
   for r = 1, 2, 3, on random planes and on planes full of ties.
2. The oracle's backward (`or_flat2d_backward`, which the GPU matches bit for bit) equals the gradient a
   harness routes from the reference's forward VALUES (first-in-scan-order match), bit for bit.
3. Central finite differences (eps = 1e-3) of the reference's forward agree with that gradient within
   1e-3 relative at tie-free pixels (margin > 1e-2), for dilation, erosion, opening and closing.

Skipped when oracle/_ref (poutre2 compiled from its sources) is not built."""
import numpy as np
import pytest

import oracle
from oracle import ref
from tests import adjoint_ref as A

pytestmark = pytest.mark.skipif(not ref.available(), reason="oracle/_ref/libpoutre_ref.so not built")


def planes(seed, shape, ties=False):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape).astype(np.float32)
    if ties:
        x = np.round(x * 2).astype(np.float32) / 2  # few distinct values: many tied windows
    return x


@pytest.mark.parametrize("r", [1, 2, 3])
@pytest.mark.parametrize("dilate", [True, False])
@pytest.mark.parametrize("ties", [False, True])
def test_forward_is_the_reference_forward(r, dilate, ties):
    x = planes(10 * r + ties, (3, 29, 41), ties)
    got = oracle.flat2d_forward(x, r, dilate)
    for p in range(x.shape[0]):
        np.testing.assert_array_equal(got[p], A.ref_flat(x[p], r, dilate))
        np.testing.assert_array_equal(got[p], ref.erode_dilate_nl(x[p], A.square_offsets(r), dilate))


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (6, 1), (2, 3), (64, 64)])
def test_forward_degenerate_shapes(shape):
    x = planes(3, shape)
    for dilate in (True, False):
        np.testing.assert_array_equal(oracle.flat2d_forward(x, 2, dilate), A.ref_flat(x, 2, dilate))


@pytest.mark.parametrize("r", [1, 2, 3])
@pytest.mark.parametrize("op", A.OPS)
@pytest.mark.parametrize("ties", [False, True])
def test_backward_is_routed_from_the_reference_forward(r, op, ties):
    x = planes(100 + r + ties, (33, 47), ties)
    g = planes(200 + r, (33, 47))
    exp = A.routed_chain(x, g, r, op)
    if op in ("dilation", "erosion"):
        got = oracle.flat2d_backward(x, g, r, op == "dilation")
    else:
        first_dilate = op == "closing"
        mid = oracle.flat2d_forward(x, r, first_dilate)
        got = oracle.flat2d_backward(x, oracle.flat2d_backward(mid, g, r, not first_dilate), r, first_dilate)
    np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("op", A.OPS)
def test_finite_differences_of_the_reference_forward(op):
    x = planes(7, (40, 40))
    g = planes(8, (40, 40))
    grad = A.routed_chain(x, g, 2, op)
    n = A.fd_check(x, g, 2, op, grad)
    assert n >= 100, f"only {n} tie-free pixels"
