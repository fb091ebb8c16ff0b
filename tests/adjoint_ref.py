"""Checkers for the flat-morphology adjoint built on poutre2's own forward.

The forward of a flat dilation / erosion of a float32 image by the (2r+1) x (2r+1) square is
poutre2's ``Dilate/Erode(F32 image, SESquare2D, iter=r)`` (src/low_level_morpho/ero_dil_static.cpp:229-306):
iterating the 3x3 square r times under the clipped border is the (2r+1)^2 square.  Opening is
dilate(erode(x)), closing erode(dilate(x)), each step a reference call.

* ``routed_gradient``: the gradient a harness derives from the reference's forward VALUES: each
  output pixel p sends grad_out[p] to the first window offset, in row-major order (dy, then dx),
  whose input equals the reference's output at p; contributions are summed per input pixel in
  raster order of the outputs (float32, as the GPU and the oracle sum them).
* ``fd_check``: central finite differences (eps = 1e-3) of L(x) = sum(g * F_ref(x)) at the pixels
  whose every relevant window extremum is unique by a margin > 1e-2, against a given gradient.
"""
import numpy as np

from oracle import ref

OPS = ("dilation", "erosion", "opening", "closing")


def ref_flat(x2d, r: int, dilate: bool):
    """poutre2's own Dilate/Erode(F32, SESquare2D, r) of one float32 plane."""
    return ref.erode_dilate_static(np.ascontiguousarray(x2d, dtype=np.float32), "SESquare2D", r, dilate)


def ref_forward(x2d, r: int, op: str):
    if op == "dilation":
        return ref_flat(x2d, r, True)
    if op == "erosion":
        return ref_flat(x2d, r, False)
    if op == "opening":
        return ref_flat(ref_flat(x2d, r, False), r, True)
    return ref_flat(ref_flat(x2d, r, True), r, False)


def square_offsets(r: int):
    """The (2r+1)^2 square as a runtime neighbour list (centre first, then row-major)."""
    offs = [(dy, dx) for dy in range(-r, r + 1) for dx in range(-r, r + 1)]
    offs.remove((0, 0))
    return [(0, 0)] + offs


def routed_gradient(x2d, y_ref, g, r: int):
    """grad_in from the reference's forward values y_ref (first-in-scan-order match)."""
    x = np.asarray(x2d, dtype=np.float32)
    H, W = x.shape
    arg = np.full((H, W), -1, dtype=np.int64)
    yy, xx = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    for dy in range(-r, r + 1):
        for dx in range(-r, r + 1):
            sy, sx = yy + dy, xx + dx
            inside = (sy >= 0) & (sy < H) & (sx >= 0) & (sx < W)
            sy, sx = np.clip(sy, 0, H - 1), np.clip(sx, 0, W - 1)
            hit = inside & (arg < 0) & (x[sy, sx] == y_ref)
            arg[hit] = (sy * W + sx)[hit]
    assert (arg >= 0).all(), "reference forward value not found in its window"
    gin = np.zeros(H * W, dtype=np.float32)
    np.add.at(gin, arg.ravel(), np.asarray(g, dtype=np.float32).ravel())  # raster order of the outputs
    return gin.reshape(H, W)


def routed_chain(x2d, g, r: int, op: str):
    """The routed gradient of any of OPS, each step routed on the reference's own forward."""
    if op in ("dilation", "erosion"):
        return routed_gradient(x2d, ref_forward(x2d, r, op), g, r)
    first_dilate = op == "closing"
    mid = ref_flat(x2d, r, first_dilate)
    out = ref_flat(mid, r, not first_dilate)
    g_mid = routed_gradient(mid, out, g, r)
    return routed_gradient(x2d, mid, g_mid, r)


def _window_gap(x, r: int, dilate: bool):
    """Per output pixel: the distance from its window's extremum to the nearest DIFFERENT value of the
    clipped window (inf when the window holds one value).  Equal values at the top are allowed: in the
    second stage of an opening they are copies of one input pixel (a plateau of the erosion), which a
    change of that pixel moves together."""
    H, W = x.shape
    pad = np.pad(x.astype(np.float64), r, constant_values=np.nan)
    stack = np.stack([pad[r + dy:r + dy + H, r + dx:r + dx + W]
                      for dy in range(-r, r + 1) for dx in range(-r, r + 1)])
    if dilate:
        stack = np.where(np.isnan(stack), -np.inf, stack)
        best = stack.max(axis=0)
        other = np.where(stack < best, stack, -np.inf).max(axis=0)
        gap = best - other
    else:
        stack = np.where(np.isnan(stack), np.inf, stack)
        best = stack.min(axis=0)
        other = np.where(stack > best, stack, np.inf).min(axis=0)
        gap = other - best
    return np.where(np.isfinite(gap), gap, np.inf)


def _min_filter(a, k: int):
    H, W = a.shape
    pad = np.pad(a, k, constant_values=np.inf)
    return np.min(np.stack([pad[k + dy:k + dy + H, k + dx:k + dx + W]
                            for dy in range(-k, k + 1) for dx in range(-k, k + 1)]), axis=0)


def tie_free(x2d, r: int, op: str, margin: float = 1e-2):
    """Mask of the pixels q whose finite difference is well defined: every window extremum that a
    change of x[q] by eps can reach is unique by more than `margin`."""
    x = np.asarray(x2d, dtype=np.float32)
    # equal values inside a window must be copies of one input pixel: the input holds no duplicates
    assert np.unique(x).size == x.size, "finite differences need an input without repeated values"
    if op in ("dilation", "erosion"):
        return _min_filter(_window_gap(x, r, op == "dilation"), r) > margin
    first_dilate = op == "closing"
    mid = ref_flat(x, r, first_dilate)
    ok1 = _min_filter(_window_gap(x, r, first_dilate), r) > margin
    ok2 = _min_filter(_window_gap(mid, r, not first_dilate), 2 * r) > margin
    return ok1 & ok2


def fd_check(x2d, g, r: int, op: str, grad, eps: float = 1e-3, rtol: float = 1e-3, max_points=None, seed=0):
    """Central differences of sum(g * F_ref(x)) against `grad` at tie-free pixels; returns the count checked."""
    x = np.asarray(x2d, dtype=np.float32)
    g64 = np.asarray(g, dtype=np.float64)
    pts = np.argwhere(tie_free(x, r, op))
    if max_points is not None and len(pts) > max_points:
        pts = pts[np.random.default_rng(seed).permutation(len(pts))[:max_points]]

    def loss(xx):
        return float((ref_forward(xx, r, op).astype(np.float64) * g64).sum())

    for qy, qx in pts:
        xp, xm = x.copy(), x.copy()
        xp[qy, qx] = np.float32(x[qy, qx] + eps)
        xm[qy, qx] = np.float32(x[qy, qx] - eps)
        fd = (loss(xp) - loss(xm)) / (2 * eps)
        an = float(grad[qy, qx])
        assert abs(fd - an) <= rtol * max(1.0, abs(fd)), (op, int(qy), int(qx), fd, an)
    return len(pts)
