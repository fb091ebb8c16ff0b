"""The saved-arg adjoint (pg_flat_morph2d_forward_arg / _backward_arg): the forward writes one arg code
per pixel and the backward gathers from the codes alone.  Its outputs must be bit-identical to the
forward and to the recomputing backward (pg_flat_morph2d_forward / _backward), which are pinned to
the oracle and to poutre2's forward elsewhere, on tie-heavy inputs (few distinct values, so that the
first-in-scan-order rule decides), at image borders and for every square window it serves."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _inputs(shape, seed, levels):
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randint(0, levels, shape, device="cuda", generator=g).float() * 0.5 - 1.0 if levels else \
        torch.randn(shape, device="cuda", generator=g)
    gy = torch.randn(shape, device="cuda", generator=g)
    return x, gy


@pytest.mark.parametrize("r", [1, 2, 3])
@pytest.mark.parametrize("dilate", [True, False])
def test_saved_arg_equals_recomputed_arg(r, dilate):
    from poutre2_gb300 import autograd as ag
    for shape, levels in (((2, 3, 37, 70), 3), ((1, 1, 1, 5), 2), ((1, 2, 64, 64), 0), ((3, 1, 130, 61), 4),
                          ((1, 1, 33, 200), 0)):
        x, gy = _inputs(shape, r * 10 + len(shape) + levels, levels)
        y_ref = ag.flat_forward(x, r, dilate)
        y, code = ag.flat_forward_arg(x, r, dilate)
        assert torch.equal(y, y_ref), (shape, levels)
        assert int(code.max()) < (2 * r + 1) ** 2
        g_ref = ag.flat_backward(x, gy, r, dilate)
        g = ag.flat_backward_arg(code, gy, r)
        assert torch.equal(g, g_ref), (shape, levels)


@pytest.mark.parametrize("op", ["dilation", "erosion", "opening", "closing"])
def test_autograd_saved_arg_matches_the_oracle(op):
    from poutre2_gb300 import autograd as ag
    x, gy = _inputs((2, 2, 45, 52), 17, 5)
    xr = x.clone().requires_grad_(True)
    out = getattr(ag, op)(xr, 2)
    out.backward(gy)
    xh, gh = x.cpu().numpy().astype(np.float32), gy.cpu().numpy().astype(np.float32)
    dil = op in ("dilation", "closing")
    exp_g = np.empty_like(xh)
    for i in range(xh.shape[0]):
        for j in range(xh.shape[1]):
            if op in ("dilation", "erosion"):
                exp_g[i, j] = oracle.flat2d_backward(xh[i, j], gh[i, j], 2, dil)
            else:
                first = op == "closing"
                mid = oracle.flat2d_forward(xh[i, j], 2, first)
                gm = oracle.flat2d_backward(mid, gh[i, j], 2, not first)
                exp_g[i, j] = oracle.flat2d_backward(xh[i, j], gm, 2, first)
    np.testing.assert_array_equal(xr.grad.cpu().numpy(), exp_g)


def test_saved_arg_rejects_other_windows():
    from poutre2_gb300 import _lib
    x = torch.zeros((1, 1, 8, 8), device="cuda")
    y, c = torch.empty_like(x), torch.empty(x.shape, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    L = _lib.load()
    assert L.pg_flat_morph2d_forward_arg(x.data_ptr(), y.data_ptr(), c.data_ptr(), 1, 8, 8, 4, 1, s) == 1
    assert L.pg_flat_morph2d_backward_arg(c.data_ptr(), x.data_ptr(), y.data_ptr(), 1, 8, 8, 0, s) == 1
    assert L.pg_flat_morph2d_backward_arg(c.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 8, 8, 2, s) == 5
