"""The CUDA path against poutre2 ITSELF at the benchmark workloads' full sizes.

The reference is poutre2's own code compiled from its sources into oracle/_ref/libpoutre_ref.so and
called through its public API (Dilate/Erode, DilateX/Y, ErodeX/Y, geo::h_maxima + CompareImage,
geo::leveling, neighbour-list Dilate/Erode).  Bit-exact throughout (tolerance 0).  Where the reference
cannot express a case directly the comparison follows its composition rules: uint16 images run on its
int32 path (widened, then narrowed: min/max commute with the monotone embedding); opening = Dilate of
Erode, closing = Erode of Dilate, gradient = Dilate - Erode (plain subtraction); the 31x31 square is
Dilate(SESquare2D, 15); the 63-pixel segments are DilateX/Y(31) and the neighbour list (-t, +t); the
3x3x3 cube is the neighbour-list path with poutre::se::SESquare3D (its slice-wise static path mixes
slices on random volumes, see test_oracle_vs_reference.py).

Skipped when oracle/_ref was not built."""
import numpy as np
import pytest
import torch

from oracle import ref
from poutre2_gb300 import synthetic

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref.available(), reason="oracle/_ref/libpoutre_ref.so not built")]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def widen(a):
    """Reference input for a pixel type it lacks (uint16 -> int32)."""
    return a.astype(np.int32) if a.dtype == np.uint16 else a


def narrow(r, dt):
    return r.astype(dt)


def test_cfg1_plain_512_u8():
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    f = synthetic.uniform_u8((512, 512), 0)
    x = dev(f)
    for se in ("SESquare2D", "SECross2D"):
        for dil in (True, False):
            out = torch.empty_like(x)
            (llm.Dilate if dil else llm.Erode)(x, Common_NL_SE[se], 1, out)
            np.testing.assert_array_equal(host(out), ref.erode_dilate_static(f, se, 1, dil), err_msg=se)


@pytest.mark.parametrize("size", [2048, 4096])
def test_cfg2_h_maxima(size):
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    f = synthetic.smoothed_noise_u8((size, size), 1, 4.0)
    x = dev(f)
    out = torch.empty_like(x)
    geo.h_maxima_binary(x, 20, Common_NL_SE.SESquare2D, out)
    np.testing.assert_array_equal(host(out), ref.h_maxima_binary(f, 20, "SESquare2D"))
    rec = torch.empty_like(x)
    geo.h_maxima(x, 20, Common_NL_SE.SESquare2D, rec)
    np.testing.assert_array_equal(host(rec), ref.extrema("h_maxima", f, 20, "SESquare2D"))


def test_cfg2_leveling_2048():
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    f = synthetic.smoothed_noise_u8((2048, 2048), 1, 4.0)
    m = synthetic.leveling_marker(f, 16.0)
    out = torch.empty_like(dev(f))
    geo.leveling(dev(f), dev(m), Common_NL_SE.SESquare2D, out)
    np.testing.assert_array_equal(host(out), ref.leveling("leveling", f, m, "SESquare2D"))


def _cfg3_image(dt):
    if dt == "u16":
        return synthetic.uniform_u16((4096, 4096), 2)
    if dt == "i32":  # the u16 workload's values on the reference's own int32 type
        return synthetic.uniform_u16((4096, 4096), 2).astype(np.int32)
    return synthetic.normal_f32((4096, 4096), 3)


@pytest.mark.parametrize("dt", ["u16", "i32", "f32"])
def test_cfg3_square_31_and_composites(dt):
    from poutre2_gb300 import llm
    a = _cfg3_image(dt)
    w = widen(a)
    x = dev(a)
    out = torch.empty_like(x)
    d = narrow(ref.erode_dilate_static(w, "SESquare2D", 15, True), a.dtype)
    e = narrow(ref.erode_dilate_static(w, "SESquare2D", 15, False), a.dtype)
    cases = [(llm.DilateSE, d), (llm.ErodeSE, e), (llm.Gradient, (d - e).astype(a.dtype)),
             (llm.Opening, narrow(ref.erode_dilate_static(widen(e), "SESquare2D", 15, True), a.dtype)),
             (llm.Closing, narrow(ref.erode_dilate_static(widen(d), "SESquare2D", 15, False), a.dtype))]
    for fn, exp in cases:
        fn(x, llm.se_rect(15, 15), out)
        np.testing.assert_array_equal(host(out), exp, err_msg=fn.__name__)
    # the reference's own call form: Dilate(SESquare2D, iter = 15)
    from poutre2_gb300.se import Common_NL_SE
    llm.Dilate(x, Common_NL_SE.SESquare2D, 15, out)
    np.testing.assert_array_equal(host(out), d)


@pytest.mark.parametrize("dt", ["u16", "i32", "f32"])
def test_cfg3_segments_63(dt):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import NeighborList
    a = _cfg3_image(dt)
    w = widen(a)
    x = dev(a)
    out = torch.empty_like(x)
    for dil in (True, False):
        exp_x = narrow(ref.line(w, 31, "x", dil), a.dtype)
        exp_y = narrow(ref.line(w, 31, "y", dil), a.dtype)
        (llm.DilateX if dil else llm.ErodeX)(x, 31, out)
        np.testing.assert_array_equal(host(out), exp_x)
        (llm.DilateY if dil else llm.ErodeY)(x, 31, out)
        np.testing.assert_array_equal(host(out), exp_y)
        seg = NeighborList.segment(-1, 1, 31)
        exp_d = narrow(ref.erode_dilate_nl(w, seg.offsets, dil), a.dtype)
        (llm.DilateSE if dil else llm.ErodeSE)(x, llm.se_line(-1, 1, 31), out)
        np.testing.assert_array_equal(host(out), exp_d)
    # openings / closings / gradients by the three segments, each a composition of reference calls
    for se, fwd in ((llm.se_line(0, 1, 31), lambda v, dl: ref.line(v, 31, "x", dl)),
                    (llm.se_line(1, 0, 31), lambda v, dl: ref.line(v, 31, "y", dl)),
                    (llm.se_line(-1, 1, 31), lambda v, dl: ref.erode_dilate_nl(v, NeighborList.segment(-1, 1, 31).offsets, dl))):
        d, e = fwd(w, True), fwd(w, False)
        for fn, exp in ((llm.Opening, fwd(e, True)), (llm.Closing, fwd(d, False)), (llm.Gradient, d - e)):
            fn(x, se, out)
            np.testing.assert_array_equal(host(out), narrow(exp, a.dtype), err_msg=fn.__name__)


def test_cfg3_cube_256():
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE, predefined_offsets
    v = synthetic.uniform_u8((256, 256, 256), 4)
    x = dev(v)
    for dil in (True, False):
        out = torch.empty_like(x)
        (llm.Dilate if dil else llm.Erode)(x, Common_NL_SE.SESquare3D, 1, out)
        np.testing.assert_array_equal(host(out), ref.erode_dilate_nl(v, predefined_offsets("SESquare3D"), dil))


def test_cfg4_ragged_batch_subset():
    """The first 64 images of the 512-image ragged batch, run as one batch."""
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    imgs = synthetic.ragged_batch(512, 5, 4.0)[:64]
    xs = [dev(f) for f in imgs]
    outs = [torch.empty_like(x) for x in xs]
    geo.h_maxima_binary_batch(xs, 10, Common_NL_SE.SESquare2D, outs)
    for f, o in zip(imgs, outs):
        np.testing.assert_array_equal(host(o), ref.h_maxima_binary(f, 10, "SESquare2D"))


def test_cfg5_planes_vs_reference_forward():
    """Two planes of the [64, 32, 256, 256] float32 tensor: the forward against poutre2's
    Dilate/Erode(F32, SESquare2D, 2), the backward against the gradient routed from those values."""
    from poutre2_gb300 import autograd
    from tests import adjoint_ref as A
    gen = torch.Generator(device="cuda").manual_seed(6)
    x = torch.randn((2, 2, 256, 256), device="cuda", generator=gen)
    g = torch.randn(x.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(7))
    xs, gs = host(x), host(g)
    for op in A.OPS:
        xt = x.clone().requires_grad_(True)
        y = getattr(autograd, op)(xt, 2)
        y.backward(g)
        yh, gh = host(y.detach()), host(xt.grad)
        for p in range(2):
            np.testing.assert_array_equal(yh[1, p], A.ref_forward(xs[1, p], 2, op), err_msg=op)
            np.testing.assert_array_equal(gh[1, p], A.routed_chain(xs[1, p], gs[1, p], 2, op), err_msg=op)
