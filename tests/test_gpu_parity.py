"""GPU parity: the CUDA path (through the C ABI) against the reference's known answers and
against the oracle on seeded random inputs.  Integer, byte and float min/max results must be
bit-exact (tolerance 0)."""
import numpy as np
import pytest
import torch

import oracle
from tests.kats import case_id, load_cases, to_array

pytestmark = pytest.mark.gpu

TYPES = [np.uint8, np.uint16, np.int32, np.int64, np.float32, np.float64]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from poutre2_gb300 import _lib
    _lib.load()
    yield


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rand(rng, shape, dt):
    dt = np.dtype(dt)
    if dt.kind == "f":
        return rng.standard_normal(shape).astype(dt)
    info = np.iinfo(dt)
    lo, hi = max(info.min, -100000), min(info.max, 100000)
    if dt == np.uint8:
        lo, hi = 0, 255
    return rng.integers(lo, hi + 1, shape, dtype=np.int64).astype(dt)


# ----------------------------------------------------------------------------- known answers
CASES = load_cases()


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_reference_kat_on_gpu(case):
    from poutre2_gb300 import geo, llm
    from poutre2_gb300.se import Common_NL_SE, NeighborList
    ins = [dev(to_array(i)) for i in case["inputs"]]
    exp = to_array(case["expected"])
    out = torch.empty_like(ins[0])
    op = case["op"]
    if op in ("dilate_static", "erode_static"):
        (llm.Dilate if op.startswith("dilate") else llm.Erode)(ins[0], Common_NL_SE[case["se"]], 1, out)
    elif op in ("dilate_nl", "erode_nl"):
        (llm.Dilate if op.startswith("dilate") else llm.Erode)(ins[0], NeighborList.predefined(case["se"]), out)
    elif op in ("dilatex", "erodex", "dilatey", "erodey"):
        fn = {"dilatex": llm.DilateX, "erodex": llm.ErodeX, "dilatey": llm.DilateY, "erodey": llm.ErodeY}[op]
        fn(ins[0], case["half"], out)
    elif op.startswith("reconstruct_"):
        geo.Reconstruction(geo.reconstruction_type.dilate if op.endswith("dilate") else geo.reconstruction_type.erode,
                           ins[0], ins[1], Common_NL_SE[case["se"]], out)
    elif op in ("low_leveling", "high_leveling", "leveling"):
        getattr(geo, op)(ins[0], ins[1], Common_NL_SE[case["se"]], out)
    elif op == "compare":
        from poutre2_gb300 import pixel
        from tests.kats import COMP_VALUES, OUT_PTYPES, compare_operands
        out = torch.empty(ins[0].shape, dtype=getattr(torch, OUT_PTYPES[case["out_ptype"]]), device="cuda")
        pixel.CompareImage(ins[0], COMP_VALUES[case["cmp"]], *compare_operands(case, ins), out)
    elif op in ("label_binary", "label_flat_zones", "label_minima", "label_maxima"):
        from poutre2_gb300 import label
        out = torch.empty(ins[0].shape, dtype=torch.int64, device=ins[0].device)
        n = getattr(label, op)(ins[0], Common_NL_SE[case["se"]], out)
        assert n == int(exp.max())
    else:
        getattr(geo, op)(ins[0], case["h"], Common_NL_SE[case["se"]], out)
    np.testing.assert_array_equal(host(out), exp)


# ----------------------------------------------------------------------------- static SEs
SHAPES_2D = [(1, 1), (1, 37), (29, 1), (5, 5), (17, 33), (64, 64), (127, 130), (256, 48)]


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("se", ["SESquare2D", "SECross2D", "SESegmentX2D", "SESegmentY2D"])
def test_static_2d_random(dt, se):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(abs(hash((se, str(dt)))) % 2**32)
    for shape in SHAPES_2D:
        a = rand(rng, shape, dt)
        x = dev(a)
        # 1-2 take the repeated 3x3 pass, the rest the line kernels (the square from 3 or 5)
        for it in (1, 2, 3, 5, 7, 40):
            for dil in (True, False):
                out = torch.empty_like(x)
                (llm.Dilate if dil else llm.Erode)(x, Common_NL_SE[se], it, out)
                np.testing.assert_array_equal(host(out), oracle.erode_dilate_static(a, se, it, dil),
                                              err_msg=f"{se} {shape} iter={it} dilate={dil}")


def test_static_unaligned_views_use_scalar_path():
    # a row width that is not a multiple of 16 bytes and a 16-byte-misaligned base
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(3)
    a = rand(rng, (40, 50), np.uint8)
    big = torch.zeros(40 * 50 + 3, dtype=torch.uint8, device="cuda")
    x = big[3:].view(40, 50)
    x.copy_(dev(a))
    out = torch.empty_like(x)
    llm.Dilate(x, Common_NL_SE.SESquare2D, 1, out)
    np.testing.assert_array_equal(host(out), oracle.dilate(a, "SESquare2D"))


@pytest.mark.parametrize("se", ["SESegmentX1D"])
@pytest.mark.parametrize("dt", TYPES)
def test_static_1d(se, dt):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(1)
    for n in (1, 2, 15, 16, 17, 1000):
        a = rand(rng, (n,), dt)
        x = dev(a)
        for it in (1, 2, 9):
            for dil in (True, False):
                out = torch.empty_like(x)
                (llm.Dilate if dil else llm.Erode)(x, Common_NL_SE[se], it, out)
                np.testing.assert_array_equal(host(out), oracle.erode_dilate_static(a, se, it, dil),
                                              err_msg=f"n={n} iter={it} dilate={dil}")


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int32, np.float32])
@pytest.mark.parametrize("se", ["SESquare3D", "SECross3D", "SESegmentX3D", "SESegmentY3D", "SESegmentZ3D"])
def test_static_3d(dt, se):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(5)
    # rows of a multiple of 16 bytes take the slice-streaming cube kernel: one slice, several tiles
    # across, down and in depth
    for shape in [(1, 1, 1), (3, 3, 3), (5, 7, 9), (17, 20, 64), (2, 33, 31), (1, 5, 16), (19, 70, 160), (9, 40, 528)]:
        a = rand(rng, shape, dt)
        x = dev(a)
        for dil in (True, False):
            out = torch.empty_like(x)
            (llm.Dilate if dil else llm.Erode)(x, Common_NL_SE[se], 1, out)
            np.testing.assert_array_equal(host(out), oracle.erode_dilate_static(a, se, 1, dil), err_msg=f"{shape}")


@pytest.mark.parametrize("cse,rank", [("Octagon", 2), ("Rhombicuboctahedron", 3)])
def test_compound(cse, rank):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Compound_NL_SE
    rng = np.random.default_rng(8)
    shape = (40, 45) if rank == 2 else (12, 13, 14)
    a = rand(rng, shape, np.int32)
    x = dev(a)
    cross, square = ("SECross2D", "SESquare2D") if rank == 2 else ("SECross3D", "SESquare3D")
    for size in (0, 2, 3, 5, 8):
        out = torch.empty_like(x)
        llm.Dilate(x, Compound_NL_SE[cse], size, out)
        nb = size / (1 + 2 ** 0.5)
        nsq = int(np.floor(nb) if nb - np.floor(nb) < 0.5 else np.floor(nb) + 1)
        exp = a.copy()
        for p in ([cross] * (size - nsq) + [square] * nsq) if size else []:
            exp = oracle.dilate(exp, p, 1)
        np.testing.assert_array_equal(host(out), exp, err_msg=f"size={size}")


@pytest.mark.parametrize("dt", TYPES)
def test_octagon_sizes(dt):
    # the octagon's cross passes and fused trailing box against the oracle's passes (pinned against
    # poutre2's compound Dilate / Erode), on small, thin and ragged images
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Compound_NL_SE
    rng = np.random.default_rng(hash((str(dt), "octagon")) % 2**32)
    for shape in [(1, 1), (1, 90), (77, 1), (64, 64), (130, 67), (203, 300)]:
        a = rand(rng, shape, dt)
        x = dev(a)
        for size in (2, 3, 5, 8, 13, 16, 17):
            for dil in (True, False):
                out = torch.empty_like(x)
                (llm.Dilate if dil else llm.Erode)(x, Compound_NL_SE.Octagon, size, out)
                np.testing.assert_array_equal(host(out), oracle.erode_dilate_compound(a, "Octagon", size, dil),
                                              err_msg=f"{shape} size={size} dilate={dil}")


# ----------------------------------------------------------------------------- neighbour lists, lines
@pytest.mark.parametrize("dt", TYPES)
def test_neighbor_list(dt):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import NeighborList
    rng = np.random.default_rng(2)
    a = rand(rng, (45, 70), dt)
    x = dev(a)
    for nl in (NeighborList.segment(-1, 1, 7), NeighborList.rectangle(2, 2), NeighborList([(0, 3), (-2, -1)])):
        for dil in (True, False):
            out = torch.empty_like(x)
            (llm.Dilate if dil else llm.Erode)(x, nl, out)
            np.testing.assert_array_equal(host(out), oracle.erode_dilate_nl(a, nl.offsets, dil))


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("half", [1, 2, 7, 31, 200])
def test_lines_xy(dt, half):
    from poutre2_gb300 import llm
    rng = np.random.default_rng(half)
    for shape in [(1, 300), (37, 37), (130, 130), (132, 132), (257, 256)]:
        a = rand(rng, shape, dt)
        x = dev(a)
        for name, axis in (("X", "x"), ("Y", "y")):
            if axis == "y" and shape[0] != shape[1]:
                continue
            for dil in (True, False):
                out = torch.empty_like(x)
                getattr(llm, ("Dilate" if dil else "Erode") + name)(x, half, out)
                np.testing.assert_array_equal(host(out), oracle.line(a, half, axis, dil), err_msg=f"{name} {shape}")


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int32, np.float32, np.float64])
@pytest.mark.parametrize("d", [(0, 1), (1, 0), (-1, 1), (1, 1)])
@pytest.mark.parametrize("half", [1, 3, 5, 7, 15, 31])
def test_segments_any_direction(dt, d, half):
    from poutre2_gb300 import llm
    from poutre2_gb300.se import NeighborList
    rng = np.random.default_rng(half * 7 + d[0] * 3 + d[1])
    offs = NeighborList.segment(d[0], d[1], half).offsets
    # word-aligned rows for every pixel type (fast path) and a ragged width (fallback)
    for shape in [(77, 150), (100, 136), (9, 260), (200, 64), (3, 4), (300, 520), (150, 1032)]:
        a = rand(rng, shape, dt)
        x = dev(a)
        for dil in (True, False):
            out = torch.empty_like(x)
            (llm.DilateSE if dil else llm.ErodeSE)(x, llm.se_line(d[0], d[1], half), out)
            np.testing.assert_array_equal(host(out), oracle.erode_dilate_nl(a, offs, dil), err_msg=f"{shape}")


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.float32])
def test_rect_and_composites(dt):
    from poutre2_gb300 import llm
    rng = np.random.default_rng(4)
    a = rand(rng, (150, 172), dt)
    x = dev(a)
    # squares up to 4 run as repeated 3x3 passes, 3-pixel segments as one 3-pixel pass
    for hy, hx in ((15, 15), (0, 4), (3, 0), (2, 9), (1, 1), (2, 2), (3, 3), (4, 4), (5, 5), (0, 1), (1, 0)):
        se = llm.se_rect(hy, hx)
        d, e = oracle.rect(a, hy, hx, True), oracle.rect(a, hy, hx, False)
        for fn, exp in ((llm.DilateSE, d), (llm.ErodeSE, e), (llm.Opening, oracle.rect(e, hy, hx, True)),
                        (llm.Closing, oracle.rect(d, hy, hx, False)), (llm.Gradient, (d - e).astype(a.dtype))):
            out = torch.empty_like(x)
            fn(x, se, out)
            np.testing.assert_array_equal(host(out), exp, err_msg=f"{fn.__name__} {hy}x{hx}")


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int32, np.float32])
@pytest.mark.parametrize("k", [7, 15, 31])
@pytest.mark.parametrize("form", ["square", "x", "y"])
def test_square_one_pass(dt, k, form):
    # 15x15, 31x31 and 63x63 squares and X / Y segments on rows of a multiple of 16 bytes take the
    # shared-memory tile kernel: images smaller than a tile, several tiles across and down, a 1-row
    # image, and (fallback) a ragged row width
    from poutre2_gb300 import llm
    hy, hx = {"square": (k, k), "x": (0, k), "y": (k, 0)}[form]
    rng = np.random.default_rng(k * 11 + np.dtype(dt).itemsize)
    for shape in [(5, 8), (1, 16), (70, 40), (300, 264), (260, 1000), (131, 520), (97, 30), (40, 2064)]:
        a = rand(rng, shape, dt)
        x = dev(a)
        d, e = oracle.rect(a, hy, hx, True), oracle.rect(a, hy, hx, False)
        for dil in (True, False):
            out = torch.empty_like(x)
            (llm.DilateSE if dil else llm.ErodeSE)(x, llm.se_rect(hy, hx), out)
            np.testing.assert_array_equal(host(out), d if dil else e, err_msg=f"{shape} dilate={dil}")
        out = torch.empty_like(x)
        llm.Gradient(x, llm.se_rect(hy, hx), out)
        np.testing.assert_array_equal(host(out), (d - e).astype(a.dtype), err_msg=f"{shape} gradient")
        for fn, exp in ((llm.Opening, oracle.rect(e, hy, hx, True)), (llm.Closing, oracle.rect(d, hy, hx, False))):
            out = torch.empty_like(x)
            fn(x, llm.se_rect(hy, hx), out)
            np.testing.assert_array_equal(host(out), exp, err_msg=f"{shape} {fn.__name__}")
    import ctypes
    from poutre2_gb300 import _lib
    _lib.call("pg_check_device", ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))  # raises on a device error


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.float32])
def test_square_iterated_equals_rect_on_gpu(dt):
    # the iterated square runs as a rectangle: check it against the oracle's 15 repeated 3x3
    # passes on a size where the line kernels take their fast (streaming / word) paths
    from poutre2_gb300 import llm
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(6)
    a = rand(rng, (300, 256), dt)
    x = dev(a)
    o1, o2 = torch.empty_like(x), torch.empty_like(x)
    llm.Dilate(x, Common_NL_SE.SESquare2D, 15, o1)
    llm.DilateSE(x, llm.se_rect(15, 15), o2)
    np.testing.assert_array_equal(host(o1), oracle.erode_dilate_static(a, "SESquare2D", 15, True))
    np.testing.assert_array_equal(host(o1), host(o2))


# ----------------------------------------------------------------------------- geodesy
def smooth(rng_seed, shape, sigma=3.0):
    from poutre2_gb300 import synthetic
    return synthetic.smoothed_noise_u8(shape, rng_seed, sigma)


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("se", ["SESquare2D", "SECross2D"])
def test_reconstruction(dt, se):
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    for k, shape in enumerate([(1, 1), (1, 100), (100, 1), (63, 65), (64, 64), (200, 333)]):
        mask = smooth(k, shape).astype(dt)
        rng = np.random.default_rng(k)
        marker = (mask.astype(np.float64) - rng.integers(0, 40, shape)).astype(np.float64)
        marker = np.clip(marker, 0, None).astype(dt)
        for dil in (True, False):
            mk = marker if dil else np.minimum(mask.astype(np.float64) + 30, 255).astype(dt)
            out = torch.empty_like(dev(mask))
            geo.Reconstruction(geo.reconstruction_type.dilate if dil else geo.reconstruction_type.erode,
                               dev(mk), dev(mask), Common_NL_SE[se], out)
            np.testing.assert_array_equal(host(out), oracle.reconstruct(mk, mask, se, dil), err_msg=f"{shape} {dil}")


def test_reconstruction_long_geodesic_paths():
    # a serpentine corridor forces propagation through many tiles and rounds
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    H, W = 300, 260
    mask = np.zeros((H, W), np.uint8)
    for r in range(0, H, 4):
        mask[r, :] = 200
        c = W - 1 if (r // 4) % 2 == 0 else 0
        mask[r:r + 4, c] = 200
    marker = np.zeros_like(mask)
    marker[0, 0] = 200
    for se in ("SESquare2D", "SECross2D"):
        out = torch.empty_like(dev(mask))
        geo.Reconstruction(geo.reconstruction_type.dilate, dev(marker), dev(mask), Common_NL_SE[se], out)
        np.testing.assert_array_equal(host(out), oracle.reconstruct(marker, mask, se, True))


def test_reconstruction_1d():
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(0)
    mask = rng.integers(0, 255, 5000).astype(np.uint8)
    marker = (mask // 3).astype(np.uint8)
    out = torch.empty_like(dev(mask))
    geo.Reconstruction(geo.reconstruction_type.dilate, dev(marker), dev(mask), Common_NL_SE.SESegmentX1D, out)
    np.testing.assert_array_equal(host(out), oracle.reconstruct(marker, mask, "SESegmentX1D", True))


@pytest.mark.parametrize("kind", ["h_minima", "h_maxima", "h_convex", "h_concave", "dynamic_pseudo_opening",
                                  "dynamic_pseudo_closing"])
@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int32, np.int64])
def test_extrema(kind, dt):
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    f = smooth(11, (150, 210)).astype(dt)
    for se in ("SESquare2D", "SECross2D"):
        out = torch.empty_like(dev(f))
        getattr(geo, kind)(dev(f), 10, Common_NL_SE[se], out)
        np.testing.assert_array_equal(host(out), getattr(oracle, kind)(f, 10, se), err_msg=se)


def test_h_maxima_binary_and_batch():
    from poutre2_gb300 import geo, synthetic
    from poutre2_gb300.se import Common_NL_SE
    imgs = [synthetic.smoothed_noise_u8(hw, 100 + i) for i, hw in enumerate([(64, 64), (65, 300), (1, 5), (333, 97),
                                                                             (128, 128), (7, 700)])]
    outs = [torch.empty_like(dev(f)) for f in imgs]
    geo.h_maxima_binary_batch([dev(f) for f in imgs], 10, Common_NL_SE.SESquare2D, outs)
    for f, o in zip(imgs, outs):
        np.testing.assert_array_equal(host(o), oracle.h_maxima_binary(f, 10))
        single = torch.empty_like(o)
        geo.h_maxima_binary(dev(f), 10, Common_NL_SE.SESquare2D, single)
        np.testing.assert_array_equal(host(single), host(o))


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int64])
def test_batch_plan_autotuned_and_graph_replay(dt):
    from poutre2_gb300 import geo, synthetic
    from poutre2_gb300.se import Common_NL_SE
    imgs = [synthetic.smoothed_noise_u8(hw, 300 + i).astype(dt) for i, hw in
            enumerate([(64, 64), (130, 70), (1, 9), (200, 333), (65, 64), (97, 1)])]
    xs = [dev(f) for f in imgs]
    outs = [torch.empty(x.shape, dtype=torch.uint8, device="cuda") for x in xs]
    plan = geo.HMaximaBinaryBatch(xs, 7, Common_NL_SE.SECross2D, outs, autotune=True)
    assert plan.config["tile"] in (32, 64)
    plan.run(check=True)
    for f, o in zip(imgs, outs):
        np.testing.assert_array_equal(host(o), oracle.h_maxima_binary(f, 7, "SECross2D"))
    # the run captured in a CUDA graph and replayed reproduces the result
    for o in outs:
        o.zero_()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run()
    for o in outs:
        o.zero_()
    g.replay()
    torch.cuda.synchronize()
    for f, o in zip(imgs, outs):
        np.testing.assert_array_equal(host(o), oracle.h_maxima_binary(f, 7, "SECross2D"))
    plan.close()


def _plateau_serpentine(H, W, step):
    """A one-pixel corridor winding through the image at 100 with a 101 bump at its far end:
    the binary h-maxima (h = 1) is 255 at the bump only once 100 has travelled the whole path."""
    f = np.zeros((H, W), np.uint8)
    rows = list(range(0, H, step))
    for i, r in enumerate(rows):
        f[r, :] = 100
        if i + 1 < len(rows):
            c = W - 1 if i % 2 == 0 else 0
            f[r:rows[i + 1] + 1, c] = 100
    last = rows[-1]
    f[last, W - 1 if len(rows) % 2 == 0 else 0] = 101
    return f


@pytest.mark.parametrize("dt", TYPES)
def test_batch_plan_pinned_configs(dt):
    # tiles that reach the sweep cap yield and are revisited; every configuration gives the same
    # result, including interior-only changes after a yield
    from poutre2_gb300 import geo, synthetic
    from poutre2_gb300.se import Common_NL_SE
    imgs = [_plateau_serpentine(70, 45, 2), _plateau_serpentine(130, 97, 3), _plateau_serpentine(33, 64, 2),
            synthetic.smoothed_noise_u8((90, 120), 5), synthetic.smoothed_noise_u8((1, 77), 6)]
    imgs = [f.astype(dt) for f in imgs]
    xs = [dev(f) for f in imgs]
    for se in ("SECross2D", "SESquare2D"):
        want = [oracle.h_maxima_binary(f, 1, se) for f in imgs]
        outs = [torch.empty(x.shape, dtype=torch.uint8, device="cuda") for x in xs]
        plan = geo.HMaximaBinaryBatch(xs, 1, Common_NL_SE[se], outs, autotune=False)
        assert plan.config["tile"] == 32
        tiles = (32,) if np.dtype(dt).itemsize == 8 else (32, 64)
        for tile in tiles:
            for sweeps in (1, 4, 512):
                plan.set_config(tile, sweeps)
                for o in outs:
                    o.fill_(7)
                plan.run(check=True)
                for i, (w, o) in enumerate(zip(want, outs)):
                    np.testing.assert_array_equal(host(o), w, err_msg=f"{se} tile {tile} sweeps {sweeps} image {i}")
        with pytest.raises(Exception):
            plan.set_config(48, 4)
        with pytest.raises(Exception):
            plan.set_config(32, 0)
        plan.close()


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("kind", ["low_leveling", "high_leveling", "leveling"])
def test_leveling(dt, kind):
    from poutre2_gb300 import geo, synthetic
    from poutre2_gb300.se import Common_NL_SE
    ref = smooth(21, (140, 190)).astype(dt)
    marker = synthetic.leveling_marker(smooth(21, (140, 190)), 6.0).astype(dt)
    for se in ("SESquare2D", "SECross2D"):
        out = torch.empty_like(dev(ref))
        getattr(geo, kind)(dev(ref), dev(marker), Common_NL_SE[se], out)
        np.testing.assert_array_equal(host(out), getattr(oracle, kind)(ref, marker, se), err_msg=se)


# ----------------------------------------------------------------------------- adjoint
@pytest.mark.parametrize("dilate", [True, False])
@pytest.mark.parametrize("r", [1, 2, 3])
def test_flat_forward_backward_exact(dilate, r):
    from poutre2_gb300 import autograd
    rng = np.random.default_rng(r)
    x = rng.standard_normal((2, 3, 37, 70)).astype(np.float32)
    x[0, 0, 5, :] = 0.5  # plateaus exercise the first-in-scan-order tie rule
    g = rng.standard_normal(x.shape).astype(np.float32)
    xt = dev(x)
    y = autograd.flat_forward(xt, r, dilate)
    np.testing.assert_array_equal(host(y), oracle.flat2d_forward(x, r, dilate))
    gx = autograd.flat_backward(xt, dev(g), r, dilate)
    np.testing.assert_array_equal(host(gx), oracle.flat2d_backward(x, g, r, dilate))


def test_opening_autograd_matches_oracle_chain():
    from poutre2_gb300 import autograd
    rng = np.random.default_rng(6)
    x = rng.standard_normal((2, 2, 40, 50)).astype(np.float32)
    g = rng.standard_normal(x.shape).astype(np.float32)
    xt = dev(x).requires_grad_(True)
    y = autograd.opening(xt, 2)
    y.backward(dev(g))
    e = oracle.flat2d_forward(x, 2, False)
    np.testing.assert_array_equal(host(y.detach()), oracle.flat2d_forward(e, 2, True))
    ge = oracle.flat2d_backward(e, g, 2, True)
    np.testing.assert_array_equal(host(xt.grad), oracle.flat2d_backward(x, ge, 2, False))


@pytest.mark.parametrize("op", ["dilation", "erosion", "opening", "closing"])
def test_gradient_vs_reference_forward(op):
    """The GPU backward against poutre2's own forward: bit-exact against the gradient routed from the
    reference's forward values, and within 1e-3 relative of central finite differences (eps = 1e-3)
    of the reference's forward at tie-free pixels (margin > 1e-2)."""
    from oracle import ref
    from poutre2_gb300 import autograd
    from tests import adjoint_ref as A
    if not ref.available():
        pytest.skip("oracle/_ref/libpoutre_ref.so not built")
    rng = np.random.default_rng(17)
    x = rng.standard_normal((1, 2, 36, 44)).astype(np.float32)
    g = rng.standard_normal(x.shape).astype(np.float32)
    xt = dev(x).requires_grad_(True)
    getattr(autograd, op)(xt, 2).backward(dev(g))
    grad = host(xt.grad)
    checked = 0
    for p in range(x.shape[1]):
        np.testing.assert_array_equal(grad[0, p], A.routed_chain(x[0, p], g[0, p], 2, op))
        checked += A.fd_check(x[0, p], g[0, p], 2, op, grad[0, p], max_points=300, seed=p)
    assert checked >= 200


# ----------------------------------------------------------------------------- errors
def test_errors_mirror_reference_checks():
    from poutre2_gb300 import geo, llm
    from poutre2_gb300._lib import PoutreError
    from poutre2_gb300.se import Common_NL_SE
    x = torch.zeros((8, 9), dtype=torch.uint8, device="cuda")
    with pytest.raises(PoutreError, match="ALIASING"):
        llm.Dilate(x, Common_NL_SE.SESquare2D, 1, x)
    with pytest.raises(PoutreError, match="INCOMPATIBLE"):
        llm.Dilate(x, Common_NL_SE.SESquare2D, 1, torch.zeros((9, 8), dtype=torch.uint8, device="cuda"))
    with pytest.raises(PoutreError, match="INCOMPATIBLE"):
        llm.Dilate(x, Common_NL_SE.SESquare2D, 1, torch.zeros((8, 9), dtype=torch.int32, device="cuda"))
    with pytest.raises(PoutreError, match="UNSUPPORTED_SE"):
        llm.Dilate(x, Common_NL_SE.SESquare3D, 1, torch.empty_like(x))
    with pytest.raises(PoutreError, match="INVALID_ARGUMENT"):
        llm.Dilate(x, Common_NL_SE.SESquare2D, -1, torch.empty_like(x))
    with pytest.raises(PoutreError, match="NOT_SQUARE"):
        llm.DilateY(x, 2, torch.empty_like(x))
    with pytest.raises(PoutreError, match="SCALAR_TYPE"):
        geo.h_maxima(x, 3.5, Common_NL_SE.SESquare2D, torch.empty_like(x))
    with pytest.raises(PoutreError, match="SCALAR_TYPE"):
        geo.h_maxima(x, -1, Common_NL_SE.SESquare2D, torch.empty_like(x))
    with pytest.raises(PoutreError, match="SCALAR_TYPE"):  # a numpy scalar keeps its type: INT32 for a UINT8 image
        geo.h_maxima(x, np.int32(3), Common_NL_SE.SESquare2D, torch.empty_like(x))
    with pytest.raises(PoutreError, match="UNSUPPORTED_SE"):
        geo.Reconstruction(geo.reconstruction_type.dilate, x, x.clone(), Common_NL_SE.SESegmentX2D, torch.empty_like(x))
    with pytest.raises(PoutreError):
        llm.Dilate(x.cpu(), Common_NL_SE.SESquare2D, 1, torch.empty_like(x))


# ----------------------------------------------------------------------------- empty images
@pytest.mark.parametrize("shape", [(0, 0), (0, 7), (5, 0)])
def test_empty_images_are_accepted(shape):
    # poutre2 images may have a zero extent; every entry point returns without computing
    from poutre2_gb300 import geo, llm
    from poutre2_gb300.se import Common_NL_SE
    x = torch.zeros(shape, dtype=torch.uint8, device="cuda")
    out = torch.zeros(shape, dtype=torch.uint8, device="cuda")
    for se in ("SESquare2D", "SECross2D", "SESegmentX2D", "SESegmentY2D"):
        llm.Dilate(x, Common_NL_SE[se], 2, out)
        llm.Erode(x, Common_NL_SE[se], 1, out)
    llm.DilateX(x, 3, out)
    llm.ErodeSE(x, llm.se_rect(2, 3), out)
    llm.DilateSE(x, llm.se_line(-1, 1, 4), out)
    llm.Opening(x, llm.se_rect(1, 1), out)
    llm.Gradient(x, llm.se_static(Common_NL_SE.SESquare2D, 1), out)
    if shape[0] == shape[1]:
        llm.DilateY(x, 2, out)
    geo.Reconstruction(geo.reconstruction_type.dilate, x, x.clone(), Common_NL_SE.SESquare2D, out)
    geo.h_maxima(x, 3, Common_NL_SE.SESquare2D, out)
    geo.h_maxima_binary(x, 3, Common_NL_SE.SESquare2D, out)
    geo.leveling(x, x.clone(), Common_NL_SE.SECross2D, out)
    y = torch.zeros((3, 4), dtype=torch.uint8, device="cuda")
    oy = torch.empty_like(y)
    geo.h_maxima_binary_batch([x, y], 3, Common_NL_SE.SESquare2D, [out, oy])
    np.testing.assert_array_equal(host(oy), oracle.h_maxima_binary(np.zeros((3, 4), np.uint8), 3, "SESquare2D"))
    torch.cuda.synchronize()


# ----------------------------------------------------------------------------- labelling
@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int32, np.int64, np.float32, np.float64])
@pytest.mark.parametrize("se,rank", [("SESquare2D", 2), ("SECross2D", 2), ("SESegmentX2D", 2), ("SESegmentY2D", 2),
                                     ("SESegmentX1D", 1), ("SECross3D", 3), ("SESegmentX3D", 3), ("SESegmentZ3D", 3)])
@pytest.mark.parametrize("flat", [False, True])
def test_labelling(dt, se, rank, flat):
    from poutre2_gb300 import label
    from poutre2_gb300.se import Common_NL_SE
    if not flat and np.dtype(dt).kind == "f":
        pytest.skip("label_binary of float images is not on the GPU path")
    rng = np.random.default_rng(abs(hash((str(dt), se, flat))) % 2**32)
    shapes = {1: [(1,), (50,), (5000,)], 2: [(1, 1), (17, 33), (130, 257)], 3: [(1, 1, 1), (6, 7, 9), (20, 33, 40)]}[rank]
    for shape in shapes:
        if flat:
            a = rng.integers(0, 3, shape).astype(dt)
        else:
            fg = rng.random(shape) < 0.5
            vals = rng.integers(-2 if np.dtype(dt).kind == "i" else 1, 5, shape)
            a = (fg * vals).astype(dt)
        out = torch.empty(shape, dtype=torch.int64, device="cuda")
        n = (label.label_flat_zones if flat else label.label_binary)(dev(a), Common_NL_SE[se], out)
        exp, m = oracle.label(a, se, flat)
        assert n == m, shape
        np.testing.assert_array_equal(host(out), exp, err_msg=f"{shape}")


def test_labelling_of_h_maxima_2048():
    # the binary h-maxima of the headline image, labelled: many components of every size
    from poutre2_gb300 import geo, label, synthetic
    from poutre2_gb300.se import Common_NL_SE
    f = synthetic.smoothed_noise_u8((2048, 2048), 1, 4.0)
    x = dev(f)
    b = torch.empty_like(x)
    geo.h_maxima_binary(x, 20, Common_NL_SE.SESquare2D, b)
    for se in ("SESquare2D", "SECross2D"):
        out = torch.empty(x.shape, dtype=torch.int64, device="cuda")
        n = label.label_binary(b, Common_NL_SE[se], out)
        exp, m = oracle.label(host(b), se, False)
        assert n == m and n > 100
        np.testing.assert_array_equal(host(out), exp)
    out = torch.empty(x.shape, dtype=torch.int64, device="cuda")
    n = label.label_flat_zones(x, Common_NL_SE.SESquare2D, out)
    exp, m = oracle.label(f, "SESquare2D", True)
    assert n == m
    np.testing.assert_array_equal(host(out), exp)


@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.int32, np.int64])
@pytest.mark.parametrize("se", ["SESquare2D", "SECross2D", "SESegmentX1D"])
@pytest.mark.parametrize("maxima", [False, True])
def test_label_extrema(dt, se, maxima):
    # label_minima / label_maxima (label_binary of h_concave / h_convex with h = 1) on plateau-rich
    # images, where regional extrema are flat zones of many shapes
    from poutre2_gb300 import label
    from poutre2_gb300.se import Common_NL_SE
    rng = np.random.default_rng(hash((str(dt), se, maxima)) % 2**32)
    shapes = [(1,), (77,), (4099,)] if se.endswith("1D") else [(1, 1), (19, 23), (200, 333)]
    for shape in shapes:
        a = rng.integers(0, 6, shape).astype(dt)
        out = torch.empty(shape, dtype=torch.int64, device="cuda")
        n = (label.label_maxima if maxima else label.label_minima)(dev(a), Common_NL_SE[se], out)
        exp, m = oracle.label_extrema(a, se, maxima)
        assert n == m, shape
        np.testing.assert_array_equal(host(out), exp, err_msg=f"{shape}")


def test_label_extrema_2048():
    from poutre2_gb300 import label, synthetic
    from poutre2_gb300.se import Common_NL_SE
    f = synthetic.smoothed_noise_u8((2048, 2048), 1, 4.0)
    x = dev(f)
    for maxima in (False, True):
        out = torch.empty(x.shape, dtype=torch.int64, device="cuda")
        n = (label.label_maxima if maxima else label.label_minima)(x, Common_NL_SE.SESquare2D, out)
        exp, m = oracle.label_extrema(f, "SESquare2D", maxima)
        assert n == m and n > 100
        np.testing.assert_array_equal(host(out), exp)


def test_labelling_rejects_like_the_reference():
    from poutre2_gb300 import label
    from poutre2_gb300._lib import PoutreError
    from poutre2_gb300.se import Common_NL_SE
    x = dev(np.ones((8, 8), np.uint8))
    with pytest.raises(PoutreError):
        label.label_binary(x, Common_NL_SE.SESquare2D, torch.empty_like(x))  # output must be int64
    with pytest.raises(PoutreError):
        label.label_binary(x, Common_NL_SE.SECross3D, torch.empty(8, 8, dtype=torch.int64, device="cuda"))
    v = dev(np.ones((4, 4, 4), np.uint8))
    with pytest.raises(PoutreError):
        label.label_binary(v, Common_NL_SE.SESquare3D, torch.empty(4, 4, 4, dtype=torch.int64, device="cuda"))


# ----------------------------------------------------------------------------- pixel processing
def _full(rng, dt, shape):
    dt = np.dtype(dt)
    if dt.kind in "iu":
        info = np.iinfo(dt)
        a = rng.integers(info.min, info.max, shape, dtype=dt, endpoint=True)
        a.reshape(-1)[:4] = [info.min, info.max, info.min, info.max][: a.size]
        return a
    return (rng.standard_normal(shape) * 1e3).astype(dt)


def _misaligned(a):
    """A device copy of ``a`` that starts one pixel into its allocation (not 16-byte aligned)."""
    buf = torch.empty(a.size + 1, dtype=getattr(torch, a.dtype.name), device="cuda")
    v = buf[1:].view(a.shape)
    v.copy_(torch.from_numpy(a))
    return v


PIXEL_SHAPES = [(1,), (17,), (5, 7), (64, 129), (3, 5, 33), (1023, 1031)]


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("kind", ["invert", "sup", "inf", "sat_add", "sat_sub"])
def test_pixel_arith(dt, kind):
    from poutre2_gb300 import pixel
    fn = {"invert": pixel.ArithInvertImage, "sup": pixel.ArithSupImage, "inf": pixel.ArithInfImage,
          "sat_add": pixel.ArithSaturatedAddImage, "sat_sub": pixel.ArithSaturatedSubImage}[kind]
    ora = {"invert": lambda a, b: oracle.invert_image(a), "sup": oracle.sup_image, "inf": oracle.inf_image,
           "sat_add": oracle.sat_add_image, "sat_sub": oracle.sat_sub_image}[kind]
    rng = np.random.default_rng(hash((str(dt), kind, "gpu")) % 2**32)
    for shape in PIXEL_SHAPES:
        a, b = _full(rng, dt, shape), _full(rng, dt, shape)
        if b.size >= 4:
            b.reshape(-1)[:4] = b.reshape(-1)[[1, 0, 0, 1]]  # (min, max), (max, min), (min, min), (max, max)
        exp = ora(a, b)
        for mis in (False, True):
            da, db = (_misaligned(a), _misaligned(b)) if mis else (dev(a), dev(b))
            out = torch.empty_like(da)
            (fn(da, out) if kind == "invert" else fn(da, db, out))
            np.testing.assert_array_equal(host(out), exp, err_msg=f"{kind} {shape} misaligned={mis}")
        da = dev(a)  # in place: the output is the first input
        (fn(da, da) if kind == "invert" else fn(da, dev(b), da))
        np.testing.assert_array_equal(host(da), exp, err_msg=f"{kind} {shape} in place")


@pytest.mark.parametrize("dt_in", TYPES)
@pytest.mark.parametrize("dt_out", TYPES)
def test_compare_all_overloads(dt_in, dt_out):
    from poutre2_gb300 import pixel
    from tests.kats import COMP_VALUES
    rng = np.random.default_rng(hash((str(dt_in), str(dt_out), "gpu")) % 2**32)
    forms = ["sss", "ssi", "sis", "sii", "iss", "isi", "iis", "iii"]
    ops = list(COMP_VALUES)
    for j, form in enumerate(forms):
        shape = [(1,), (33,), (7, 9), (130, 67), (4, 3, 21)][j % 5]
        a = rng.integers(0, 4, shape).astype(dt_in)
        opnds, dev_opnds = [], []
        for kind, dt in zip(form, (dt_in, dt_out, dt_out)):
            if kind == "i":
                v = rng.integers(0, 4, shape).astype(dt)
                opnds.append(v)
                dev_opnds.append(dev(v))
            else:
                v = int(rng.integers(0, 4))
                opnds.append(v)
                dev_opnds.append(v)
        for op in (ops[j % 6], ops[(j + 3) % 6]):
            out = torch.empty(shape, dtype=getattr(torch, np.dtype(dt_out).name), device="cuda")
            pixel.CompareImage(dev(a), COMP_VALUES[op], *dev_opnds, out)
            np.testing.assert_array_equal(host(out), oracle.compare(a, op, *opnds, dt_out), err_msg=f"{op} {form}")


def test_compare_misaligned_and_in_place():
    from poutre2_gb300 import pixel
    rng = np.random.default_rng(44)
    a = rng.integers(0, 255, (301, 257)).astype(np.uint8)
    t = rng.integers(0, 255, (301, 257)).astype(np.uint8)
    exp = oracle.compare(a, "sup", 100, t, 0, np.uint8)
    out = torch.empty(a.shape, dtype=torch.uint8, device="cuda")
    pixel.CompareImage(_misaligned(a), pixel.CompOpType.CompOpSup, 100, _misaligned(t), 0, out)
    np.testing.assert_array_equal(host(out), exp)
    da = dev(a)
    pixel.CompareImage(da, pixel.CompOpType.CompOpSup, 100, dev(t), 0, da)
    np.testing.assert_array_equal(host(da), exp)


@pytest.mark.parametrize("dt_in", TYPES)
@pytest.mark.parametrize("dt_out", TYPES)
def test_convert(dt_in, dt_out):
    from poutre2_gb300 import pixel
    rng = np.random.default_rng(hash((str(dt_in), str(dt_out), "gpu")) % 2**32)
    unsigned = np.dtype(dt_in).kind == "u" or np.dtype(dt_out).kind == "u"
    small = np.uint8 in (dt_in, dt_out)
    lo, hi = (0 if unsigned else -1000), (255 if small else 1000)
    for shape in [(1,), (19,), (33, 65), (2, 3, 17)]:
        a = rng.uniform(lo, hi, shape).astype(dt_in)
        for mis in (False, True):
            out = torch.empty(shape, dtype=getattr(torch, np.dtype(dt_out).name), device="cuda")
            pixel.ConvertInto(_misaligned(a) if mis else dev(a), out)
            np.testing.assert_array_equal(host(out), oracle.convert(a, dt_out), err_msg=f"{shape} {mis}")
    if np.dtype(dt_in).kind in "iu" and np.dtype(dt_out).kind in "iu":  # modular narrowing
        w = _full(rng, dt_in, (33, 17))
        out = torch.empty(w.shape, dtype=getattr(torch, np.dtype(dt_out).name), device="cuda")
        pixel.ConvertInto(dev(w), out)
        np.testing.assert_array_equal(host(out), oracle.convert(w, dt_out))


def test_copy_into_and_rejections():
    from poutre2_gb300 import pixel
    from poutre2_gb300._lib import PoutreError
    a = dev(np.arange(60, dtype=np.int32).reshape(6, 10))
    o = torch.empty_like(a)
    pixel.CopyInto(a, o)
    assert torch.equal(a, o)
    with pytest.raises(PoutreError):
        pixel.CopyInto(a, torch.empty(6, 10, dtype=torch.int64, device="cuda"))  # type differs
    with pytest.raises(PoutreError):
        pixel.ConvertInto(a, a.view(torch.float32))  # ConvertInto images must be different
    buf = torch.zeros(70, dtype=torch.int32, device="cuda")
    with pytest.raises(PoutreError):  # a partial overlap of output and input
        pixel.ArithSupImage(buf[:60].view(6, 10), a, buf[5:65].view(6, 10))
    with pytest.raises(PoutreError):  # the comparand must have the input's type
        pixel.CompareImage(a, pixel.CompOpType.CompOpSup, a.to(torch.int64), 1, 0, o)
    with pytest.raises(PoutreError):  # a scalar that the pixel type cannot hold
        pixel.CompareImage(a, pixel.CompOpType.CompOpSup, 0.5, 1, 0, o)


def test_int64_h_crosses_the_boundary_exactly():
    """h = 2**53 + 1 on int64 pixels near 2**62: a double would round h to 2**53 and change the
    h-maxima by one at every dome; the exact pg_scalar keeps it."""
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    base = 2**62
    f = smooth(5, (90, 120)).astype(np.int64) * (2**46) + base  # h = 128 grey levels + 1
    h = 2**53 + 1
    out = torch.empty_like(dev(f))
    geo.h_maxima(dev(f), h, Common_NL_SE.SESquare2D, out)
    exact = oracle.reconstruct(f - np.int64(h), f, "SESquare2D", True)
    rounded = oracle.reconstruct(f - np.int64(float(h)), f, "SESquare2D", True)
    assert not np.array_equal(exact, rounded)
    np.testing.assert_array_equal(host(out), exact)


def test_pypoutre_names():
    # poutre2's Python names (python/*/*.cpp) on device images, end to end
    from poutre2_gb300 import pypoutre as pp
    rng = np.random.default_rng(45)
    f = rng.integers(0, 200, (37, 53)).astype(np.uint8)
    img = pp.from_numpy(f)
    assert img.ptype() == pp.PType.GrayUINT8 and img.shape() == [37, 53] and img.rank() == 2
    out = pp.clone_geometry(img)
    pp.dilate(img, pp.static_nl_se.square2d, 2, out)
    np.testing.assert_array_equal(out.numpy(), oracle.erode_dilate_static(f, "SESquare2D", 2, True))
    pp.erodeX(img, 3, out)
    np.testing.assert_array_equal(out.numpy(), oracle.line(f, 3, "x", False))
    pp.h_maxima(img, 20, pp.static_nl_se.square2d, out)
    np.testing.assert_array_equal(out.numpy(), oracle.h_maxima(f, 20, "SESquare2D"))
    pp.h_minima(img, 20, pp.static_nl_se.cross2d, out)
    np.testing.assert_array_equal(out.numpy(), oracle.h_minima(f, 20, "SECross2D"))
    marker = pp.from_numpy(oracle.sat_sub_const(f, 30))
    pp.reconstruction(pp.RecType.dilate, marker, img, pp.static_nl_se.square2d, out)
    np.testing.assert_array_equal(out.numpy(), oracle.reconstruct(oracle.sat_sub_const(f, 30), f, "SESquare2D", True))
    pp.compare(img, pp.Comp.Sup, marker, 255, 0, out)
    np.testing.assert_array_equal(out.numpy(), oracle.compare(f, "sup", oracle.sat_sub_const(f, 30), 255, 0, np.uint8))
    pp.arith_saturated_sub_image(img, marker, out)
    np.testing.assert_array_equal(out.numpy(), oracle.sat_sub_image(f, oracle.sat_sub_const(f, 30)))
    c = pp.convert(img, pp.CType.Scalar, pp.PType.GrayINT64)
    assert c.ptype() == pp.PType.GrayINT64 and np.array_equal(c.numpy(), f.astype(np.int64))
    lab = pp.factory_image([37, 53], pp.CType.Scalar, pp.PType.GrayINT64)
    assert pp.label_flat_zones(img, pp.static_nl_se.square2d, lab) == oracle.label(f, "SESquare2D", True)[1]
    pp.label_maxima(img, pp.static_nl_se.square2d, lab)
    np.testing.assert_array_equal(lab.numpy(), oracle.label_extrema(f, "SESquare2D", True)[0])
    assert pp.to_string(pp.from_string("Scalar GINT32 2 1 3 1 -2 3")) == "Scalar GINT32 2 1 3 1 -2 3"
    # an object that exports a CUDA buffer through DLPack is taken without a copy

    class Exporter:
        def __init__(self, t):
            self.t = t

        def __dlpack__(self, **kw):
            return self.t.__dlpack__(**kw)

        def __dlpack_device__(self):
            return self.t.__dlpack_device__()

    t = torch.from_numpy(f).cuda()
    o = torch.empty_like(t)
    pp.arith_invert_image(Exporter(t), Exporter(o))
    np.testing.assert_array_equal(host(o), oracle.invert_image(f))


# ----------------------------------------------------------------------------- 3D geodesy
def _volume(seed, shape, dt):
    rng = np.random.default_rng(seed)
    v = rng.integers(0, 60, shape)
    return v.astype(dt)


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("se", ["SECross3D"])
def test_reconstruction_3d(dt, se):
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    for k, shape in enumerate([(1, 1, 1), (1, 1, 40), (5, 6, 7), (20, 33, 40)]):
        mask = _volume(k, shape, dt)
        for dil in (True, False):
            mk = (mask // 2).astype(dt) if dil else (mask + 25).astype(dt)
            out = torch.empty_like(dev(mask))
            geo.Reconstruction(geo.reconstruction_type.dilate if dil else geo.reconstruction_type.erode,
                               dev(mk), dev(mask), Common_NL_SE[se], out)
            np.testing.assert_array_equal(host(out), oracle.reconstruct(mk, mask, se, dil), err_msg=f"{shape} {dil}")


def test_reconstruction_3d_long_path():
    # a corridor that winds through the slices: the fixpoint needs hundreds of steps
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    D, H, W = 8, 24, 30
    mask = np.zeros((D, H, W), np.uint8)
    for z in range(D):
        for r in range(0, H, 3):
            mask[z, r, :] = 150
            c = W - 1 if (r // 3) % 2 == 0 else 0
            mask[z, r:r + 3, c] = 150
        mask[z, H - 1 if z % 2 == 0 else 0, :] = 150
    marker = np.zeros_like(mask)
    marker[0, 0, 0] = 150
    out = torch.empty_like(dev(mask))
    geo.Reconstruction(geo.reconstruction_type.dilate, dev(marker), dev(mask), Common_NL_SE.SECross3D, out)
    np.testing.assert_array_equal(host(out), oracle.reconstruct(marker, mask, "SECross3D", True))


@pytest.mark.parametrize("kind", ["h_minima", "h_maxima", "h_convex", "h_concave", "dynamic_pseudo_opening",
                                  "dynamic_pseudo_closing"])
def test_extrema_3d(kind):
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    for dt in (np.uint8, np.int32):
        f = _volume(31, (9, 17, 23), dt)
        for se in ("SECross3D",):
            out = torch.empty_like(dev(f))
            getattr(geo, kind)(dev(f), 7, Common_NL_SE[se], out)
            np.testing.assert_array_equal(host(out), getattr(oracle, kind)(f, 7, se), err_msg=f"{se} {dt}")


@pytest.mark.parametrize("kind", ["low_leveling", "high_leveling", "leveling"])
def test_leveling_3d(kind):
    from poutre2_gb300 import geo
    from poutre2_gb300.se import Common_NL_SE
    for dt in (np.uint8, np.float32):
        ref = _volume(41, (7, 15, 19), dt)
        marker = _volume(42, (7, 15, 19), dt)
        for se in ("SECross3D",):
            out = torch.empty_like(dev(ref))
            getattr(geo, kind)(dev(ref), dev(marker), Common_NL_SE[se], out)
            np.testing.assert_array_equal(host(out), getattr(oracle, kind)(ref, marker, se), err_msg=f"{se} {dt}")


def test_h_maxima_binary_and_label_extrema_3d():
    from poutre2_gb300 import geo, label
    from poutre2_gb300.se import Common_NL_SE
    f = _volume(51, (10, 21, 26), np.uint8)
    x = dev(f)
    for se in ("SECross3D",):
        b = torch.empty_like(x)
        geo.h_maxima_binary(x, 5, Common_NL_SE[se], b)
        np.testing.assert_array_equal(host(b), oracle.h_maxima_binary(f, 5, se), err_msg=se)
    for maxima in (False, True):
        out = torch.empty(f.shape, dtype=torch.int64, device="cuda")
        n = (label.label_maxima if maxima else label.label_minima)(x, Common_NL_SE.SECross3D, out)
        exp, m = oracle.label_extrema(f, "SECross3D", maxima)
        assert n == m
        np.testing.assert_array_equal(host(out), exp)
