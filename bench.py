"""Benchmark of the GB300 morphology + geodesy path.

Headline workload (one "step"): the binary h-maxima chain of a 2048x2048 uint8 image --
white noise (seed 1), Gaussian sigma=4, rescaled to [0,255]; marker = sat_sub(mask, 20);
geodesic reconstruction by dilation, 8-connectivity, to idempotence; output mask > rec as a
binary uint8 image -- in one fused persistent launch.  Metric: Gpixel/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--extra]

--impl reference times poutre2's own CPU implementation of the same workload (oracle/_ref,
compiled from the reference sources; the C restatement if that library cannot be built) on
the host cores.  Under torchrun (N > 1) every rank runs an independent replica (the images
are independent; no collective on the data path), timing is max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Gpixel/s & %HBM peak: erode/dilate, reconstruction; ragged batch vs plain"
UNIT = "Gpixel/s"
H_VALUE = 20


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_for(key):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get(key)
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(t_local, ws, device):
    """The slowest rank's step time (the job's time); the identity on one process."""
    if ws <= 1:
        return t_local
    import torch
    import torch.distributed as dist
    tt = torch.tensor([float(t_local)], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_value(pixels_per_rank, ws, t_step):
    """Whole-job throughput of `ws` replicas, each processing `pixels_per_rank` per step, in Gpixel/s."""
    return ws * pixels_per_rank / t_step / 1e9


def workload_image(size):
    from poutre2_gb300 import synthetic
    return synthetic.smoothed_noise_u8((size, size), seed=1, sigma=4.0)


def workload_name(size):
    """The workload string of both arms' `config` (identical, so that the two lines compare)."""
    return (f"binary h-maxima (sat_sub h={H_VALUE}, reconstruction by dilation 8-conn to idempotence, "
            f"mask>rec) {size}x{size} u8 smoothed noise sigma=4 seed 1")


def host_cpu():
    """Model name and logical core count of the host CPU (the CPU baseline's machine)."""
    model = platform.processor() or ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and v.strip():
                model = v.strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.lower().startswith(("model name", "cpu part")):
                        model = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"cpu_model": model or "unknown", "nproc": os.cpu_count() or 1, "arch": platform.machine()}


# ----------------------------------------------------------------------------- CPU baseline
def cpu_hmaxima_fn():
    """poutre2's CPU binary h-maxima (oracle/_ref) or, failing that, the C restatement:
    returns (fn(image, h) -> binary image, kind)."""
    try:
        from oracle import ref
        if not ref.available():
            try:
                ref.build()
            except Exception:
                pass
        if ref.available():
            return (lambda img, h: ref.h_maxima_binary(img, h, "SESquare2D")), "reference"
    except Exception:
        pass
    import oracle
    return (lambda img, h: oracle.h_maxima_binary(img, h, "SESquare2D")), "port"


def cpu_threads():
    """Host threads for the CPU leg: every core this process may run on."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def cpu_hmaxima(f, budget_s=12.0, min_runs=1, threads=1, max_runs=50):
    """Time poutre2's CPU implementation (oracle/_ref) or, failing that, the C restatement on `f`.

    poutre2 is single-threaded, so with threads > 1 each host thread runs the whole workload on its own
    copy of the image at the same time (independent replicas, as the GPU arm's ranks are); one run is
    the wall time until every thread has finished its image.  Returns (pixels/s over all threads, kind,
    runs)."""
    import concurrent.futures
    hm, kind = cpu_hmaxima_fn()
    copies = [f.copy() for _ in range(threads)]
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:  # ctypes calls release the GIL
        def one():
            list(ex.map(lambda c: hm(c, H_VALUE), copies))
        one()  # warm
        times = []
        t_end = time.perf_counter() + budget_s
        while len(times) < min_runs or time.perf_counter() < t_end:
            t0 = time.perf_counter()
            one()
            times.append(time.perf_counter() - t0)
            if len(times) >= max_runs:
                break
    return threads * f.size / statistics.median(times), kind, len(times)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    f = workload_image(args.size)
    th = cpu_threads()
    for _ in range(args.warmup):
        cpu_hmaxima(f, budget_s=0.0, threads=th)
    steps = []
    for _ in range(args.steps):
        v, kind, runs = cpu_hmaxima(f, budget_s=0.0, threads=th)
        steps.append(th * f.size / v)
    t = statistics.mean(steps)
    value = th * f.size / t / 1e9
    v1, _, runs1 = cpu_hmaxima(f, budget_s=0.0, min_runs=3)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": workload_name(args.size), "parallelism": f"replicas x{ws}"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": th, "kind": kind, **host_cpu(),
                             "sample": f"each step: {th} host threads each run the full {args.size}^2 workload on "
                                       f"its own copy (poutre2 is single-threaded; replicas, as on the GPU arm)",
                             "single_thread_value": v1 / 1e9,
                             "build": f"g++ -O3 ({platform.machine()}; xsimd stand-in of fixed-width lane "
                                      f"loops, auto-vectorised by the compiler)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------- GPU arm
def _time_ms(fn, flush, reps=5, warm=2):
    """CUDA-event time of fn() on the current stream, L2 flushed before each rep.  A GPU-side wait of
    about 100 us is queued after the flush, so that fn's launches are already enqueued when the stream
    reaches the first event: the bracket times the device work, not the host's launch path (which for
    a 10-20 us kernel is of the same order).  The GB300's event clock advances in 2.048 us steps, so a
    single reading of a 15 us kernel is off by up to 14 %; with at least 12 reps the mean of the middle
    readings (a fifth dropped at each end) is returned, which averages the steps out -- fewer reps, the
    median."""
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    spin = 200_000  # SM cycles: ~100 us at 2 GHz
    out = []
    for _ in range(reps):
        flush_l2(flush)
        torch.cuda._sleep(spin)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        fn()
        b.record(st)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    if len(out) >= 12:
        out.sort()
        cut = len(out) // 5
        return statistics.fmean(out[cut:len(out) - cut])
    return statistics.median(out)


def extra_measurements(dev, flush, only=None, cfg5_batch=64):
    """The other workloads (parity-tested in tests/test_gpu_fullsize.py), timed the same way.
    `only`: names of the groups to run (cfg1, cfg2_4096, cfg2_leveling, cfg3, large, cfg4, cfg5, label2048,
    pixel4096, octagon4096, geodesy3d), or
    all."""
    import numpy as np
    import torch

    from poutre2_gb300 import autograd, geo, llm, synthetic
    from poutre2_gb300.se import Common_NL_SE
    peak, _ = peaks()
    res = {}

    def rec(name, ms, pixels, alg_bytes, **kw):
        d = {"ms": round(ms, 5), "Gpixel_s": pixels / ms / 1e6}
        if alg_bytes:
            d["GB_s"] = alg_bytes / ms / 1e6
            d["hbm_frac"] = d["GB_s"] / peak
        d.update(kw)
        res[name] = d

    def guard(fn):
        try:
            fn()
        except Exception as e:  # keep the headline line even if an extra fails
            res.setdefault("errors", []).append(f"{fn.__name__}: {type(e).__name__}: {e}")

    def cfg1():
        x = torch.from_numpy(synthetic.uniform_u8((512, 512), 0)).to(dev)
        o = torch.empty_like(x)
        for se in ("SESquare2D", "SECross2D"):
            for dil in (True, False):
                f = (lambda s=se, d=dil: (llm.Dilate if d else llm.Erode)(x, Common_NL_SE[s], 1, o))
                rec(f"cfg1_{'dilate' if dil else 'erode'}_{se}_512_u8", _time_ms(f, flush, 20, 5), x.numel(), 2 * x.numel())

    def cfg2_4096():
        f = synthetic.smoothed_noise_u8((4096, 4096), 1, 4.0)
        x = torch.from_numpy(f).to(dev)
        o = torch.empty_like(x)
        ms = _time_ms(lambda: geo.h_maxima_binary(x, H_VALUE, Common_NL_SE.SESquare2D, o, check=False), flush, 5, 2)
        rounds = geo.last_reconstruction_rounds()
        cpu_v, kind, runs = cpu_hmaxima(f, budget_s=0.0)  # poutre2 on one core
        cpu_ms = f.size / cpu_v * 1e3
        th = cpu_threads()  # and on every core at once (one image per thread)
        cpu_vp, _, _ = cpu_hmaxima(f, budget_s=0.0, threads=th)
        rec("cfg2_h_maxima_binary_4096_u8", ms, f.size, 2 * f.size, cpu_ms=cpu_ms, cpu_kind=kind,
            speedup_vs_cpu=cpu_ms / ms, cpu_threads=th, cpu_all_threads_gpx_s=cpu_vp / 1e9,
            speedup_vs_cpu_all_threads=(f.size / ms / 1e6) / (cpu_vp / 1e9), rounds=rounds)

    def cfg2_leveling():
        f = synthetic.smoothed_noise_u8((2048, 2048), 1, 4.0)
        m = synthetic.leveling_marker(f, 16.0)
        x, mk = torch.from_numpy(f).to(dev), torch.from_numpy(m).to(dev)
        o = torch.empty_like(x)
        ms = _time_ms(lambda: geo.leveling(x, mk, Common_NL_SE.SESquare2D, o, check=False), flush, 5, 2)
        kw = {}
        try:
            from oracle import ref
            if ref.available():
                t0 = time.perf_counter()
                ref.leveling("leveling", f, m, "SESquare2D")
                kw = {"cpu_ms": (time.perf_counter() - t0) * 1e3, "cpu_kind": "reference"}
                kw["speedup_vs_cpu"] = kw["cpu_ms"] / ms
        except Exception:
            pass
        rec("cfg2_leveling_2048_u8", ms, f.size, 3 * f.size, **kw)

    def cfg3():
        for dt, arr in (("u16", synthetic.uniform_u16((4096, 4096), 2)), ("f32", synthetic.normal_f32((4096, 4096), 3))):
            x = torch.from_numpy(arr).to(dev)
            o = torch.empty_like(x)
            es = x.element_size()
            for sname, se in (("square31", llm.se_rect(15, 15)), ("h63", llm.se_line(0, 1, 31)),
                              ("v63", llm.se_line(1, 0, 31)), ("d45_63", llm.se_line(-1, 1, 31))):
                for op, fn in (("dilate", llm.DilateSE), ("erode", llm.ErodeSE), ("opening", llm.Opening),
                               ("closing", llm.Closing), ("gradient", llm.Gradient)):
                    ms = _time_ms(lambda fn=fn, se=se: fn(x, se, o), flush, 15, 2)
                    rec(f"cfg3_{op}_{sname}_4096_{dt}", ms, x.numel(), 2 * x.numel() * es)
            del x, o
        # the 3x3 square on a 4096^2 u8 image and the 3x3x3 cube on a 256^3 u8 volume (TMA tile kernels)
        x8 = torch.from_numpy(synthetic.uniform_u8((4096, 4096), 2)).to(dev)
        o8 = torch.empty_like(x8)
        for dil in (True, False):
            ms = _time_ms(lambda d=dil: (llm.Dilate if d else llm.Erode)(x8, Common_NL_SE.SESquare2D, 1, o8), flush, 15, 3)
            rec(f"cfg3_{'dilate' if dil else 'erode'}_square3_4096_u8", ms, x8.numel(), 2 * x8.numel())
        del x8, o8
        v = torch.from_numpy(synthetic.uniform_u8((256, 256, 256), 4)).to(dev)
        o = torch.empty_like(v)
        for dil in (True, False):
            ms = _time_ms(lambda d=dil: (llm.Dilate if d else llm.Erode)(v, Common_NL_SE.SESquare3D, 1, o), flush, 15, 3)
            rec(f"cfg3_{'dilate' if dil else 'erode'}_cube3_256_u8", ms, v.numel(), 2 * v.numel())
        # the event bracket's own floor: a 16-element add timed the same way (part of every row above)
        z = torch.zeros(16, device=dev)
        res["event_floor_add16_us"] = round(_time_ms(lambda: z.add_(1), flush, 15, 3) * 1e3, 2)

    def large():
        # 16384^2 u16 (512 MiB in, 512 MiB out): the output is four times the 129 MB L2, so the
        # timed kernel pays its own DRAM write-back and the fraction is a DRAM figure
        rng = np.random.default_rng(2)
        x = torch.from_numpy(rng.integers(0, 65536, (16384, 16384), dtype=np.uint16)).to(dev)
        o = torch.empty_like(x)
        for sname, se in (("square31", llm.se_rect(15, 15)), ("h63", llm.se_line(0, 1, 31)),
                          ("v63", llm.se_line(1, 0, 31)), ("d45_63", llm.se_line(-1, 1, 31))):
            for op, fn in (("dilate", llm.DilateSE), ("opening", llm.Opening), ("gradient", llm.Gradient)):
                ms = _time_ms(lambda fn=fn, se=se: fn(x, se, o), flush, 3, 1)
                rec(f"large_{op}_{sname}_16384_u16", ms, x.numel(), 4 * x.numel())
        ms = _time_ms(lambda: llm.Dilate(x, Common_NL_SE.SESquare2D, 1, o), flush, 3, 1)
        rec("large_dilate_square3_16384_u16", ms, x.numel(), 4 * x.numel())
        del x, o

    def cfg4():
        imgs = synthetic.ragged_batch(512, 5, 4.0)
        xs = [torch.from_numpy(f).to(dev) for f in imgs]
        outs = [torch.empty_like(x) for x in xs]
        npx = sum(f.size for f in imgs)
        plan = geo.HMaximaBinaryBatch(xs, 10, Common_NL_SE.SESquare2D, outs, autotune=True)
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            plan.run()
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            plan.run()
        graph_ms = _time_ms(graph.replay, flush, 5, 2)
        plan_ms = _time_ms(plan.run, flush, 5, 2)
        one_call_ms = _time_ms(lambda: geo.h_maxima_binary_batch(xs, 10, Common_NL_SE.SESquare2D, outs, check=False),
                               flush, 5, 2)

        def plain():
            for x, o in zip(xs, outs):
                geo.h_maxima_binary(x, 10, Common_NL_SE.SESquare2D, o, check=False)
        plain_ms = _time_ms(plain, flush, 3, 1)
        kw = {}
        try:  # poutre2 on the host: one core, and the images spread over every core (harness threads)
            import concurrent.futures
            hm, kind = cpu_hmaxima_fn()
            t0 = time.perf_counter()
            for f in imgs:
                hm(f, 10)
            one = (time.perf_counter() - t0) * 1e3
            cores = os.cpu_count() or 1
            t0 = time.perf_counter()
            with concurrent.futures.ThreadPoolExecutor(cores) as ex:
                list(ex.map(lambda f: hm(f, 10), imgs))
            par = (time.perf_counter() - t0) * 1e3
            kw = {"cpu_kind": kind, "cpu_1core_ms": one, "cpu_parallel_ms": par, "cpu_parallel_threads": cores,
                  "cpu_parallel_note": "harness threads over the images; poutre2 itself is single-threaded",
                  "speedup_vs_cpu_1core": one / graph_ms, "speedup_vs_cpu_parallel": par / graph_ms}
        except Exception as e:
            kw = {"cpu_error": f"{type(e).__name__}: {e}"}
        rec("cfg4_ragged512_graph_replay", graph_ms, npx, 2 * npx, plain_ms=plain_ms,
            speedup_vs_plain=plain_ms / graph_ms, plan_run_ms=plan_ms, one_call_ms=one_call_ms,
            autotuned=plan.config, **kw)
        plan.close()

    def cfg5():
        shape = (cfg5_batch, 32, 256, 256)  # the workload's batch is 64; a smaller one only for profiling
        x = torch.randn(shape, device=dev, generator=torch.Generator(device=dev).manual_seed(6))
        g = torch.randn(shape, device=dev, generator=torch.Generator(device=dev).manual_seed(7))
        n = x.numel()
        for name, fn in (("dilation", autograd.dilation), ("erosion", autograd.erosion), ("opening", autograd.opening)):
            with torch.no_grad():
                fwd = _time_ms(lambda fn=fn: fn(x, 2), flush, 3, 1)
            xr = x.clone().requires_grad_(True)

            def fb(fn=fn):
                xr.grad = None
                fn(xr, 2).backward(g)
            fb_ms = _time_ms(fb, flush, 3, 1)
            passes = 2 if name == "opening" else 1
            tag = f"{cfg5_batch}x32x256x256"
            rec(f"cfg5_{name}_5x5_fwd_{tag}_f32", fwd, n, passes * 2 * n * 4)
            rec(f"cfg5_{name}_5x5_fwd_bwd_{tag}_f32", fb_ms, n, passes * 5 * n * 4, fwd_bwd_over_fwd=fb_ms / fwd)
            del xr

    def label2048():
        # labelling (the next row after the configs): the binary h-maxima of the headline image, and
        # the flat zones of the image itself, against poutre2 on one host core
        from poutre2_gb300 import label
        f = synthetic.smoothed_noise_u8((2048, 2048), 1, 4.0)
        x = torch.from_numpy(f).to(dev)
        b = torch.empty_like(x)
        geo.h_maxima_binary(x, H_VALUE, Common_NL_SE.SESquare2D, b)
        out = torch.empty(x.shape, dtype=torch.int64, device=dev)
        bh = b.cpu().numpy()
        for name, img, host_img, flat in (("label_binary_hmaxima", b, bh, False), ("label_flat_zones", x, f, True)):
            fn = label.label_flat_zones if flat else label.label_binary
            ms = _time_ms(lambda fn=fn, img=img: fn(img, Common_NL_SE.SESquare2D, out), flush, 5, 2)
            kw = {"note": "includes the synchronous read-back of the label count"}
            try:
                from oracle import ref
                if ref.available():
                    t0 = time.perf_counter()
                    ref.label(host_img, "SESquare2D", flat)
                    kw.update(cpu_ms=(time.perf_counter() - t0) * 1e3, cpu_kind="reference")
                    kw["speedup_vs_cpu"] = kw["cpu_ms"] / ms
            except Exception:
                pass
            rec(f"{name}_2048_u8", ms, img.numel(), img.numel() * 9, **kw)

    def pixel4096():
        # the pixel-processing kernels (HBM streams): 4096^2 u16 sup / saturated difference, the
        # h-maxima binary compare form (image comparand, scalar true / false) on u8, and a u8 -> f32
        # conversion; poutre2's own call on the host beside each
        from poutre2_gb300 import pixel
        rng = np.random.default_rng(9)
        n = 4096 * 4096
        a16 = rng.integers(0, 65536, (4096, 4096), dtype=np.uint16)
        b16 = rng.integers(0, 65536, (4096, 4096), dtype=np.uint16)
        a8 = (a16 >> 8).astype(np.uint8)
        b8 = (b16 >> 8).astype(np.uint8)
        x16, y16, o16 = (torch.from_numpy(a16).to(dev), torch.from_numpy(b16).to(dev),
                         torch.empty((4096, 4096), dtype=torch.uint16, device=dev))
        x8, y8, o8 = (torch.from_numpy(a8).to(dev), torch.from_numpy(b8).to(dev), torch.empty_like(o16, dtype=torch.uint8))
        of = torch.empty((4096, 4096), dtype=torch.float32, device=dev)
        work = (("sup_image_4096_u16", lambda: pixel.ArithSupImage(x16, y16, o16), 6 * n, "sup", (a16, b16)),
                ("sat_sub_image_4096_u16", lambda: pixel.ArithSaturatedSubImage(x16, y16, o16), 6 * n, "sat_sub",
                 (a16, b16)),
                ("compare_sup_image_4096_u8", lambda: pixel.CompareImage(x8, pixel.CompOpType.CompOpSup, y8, 255, 0, o8),
                 3 * n, "compare", (a8, b8)),
                ("convert_u8_f32_4096", lambda: pixel.ConvertInto(x8, of), 5 * n, "convert", (a8,)))
        for name, fn, nbytes, kind, host_in in work:
            ms = _time_ms(fn, flush, 20, 5)
            kw = {}
            try:
                from oracle import ref
                if ref.available():
                    h = [v.astype(np.int32) if v.dtype == np.uint16 else v for v in host_in]  # poutre2 has no u16
                    t0 = time.perf_counter()
                    if kind == "compare":
                        ref.compare(h[0], "sup", h[1], 255, 0, np.uint8)
                    elif kind == "convert":
                        ref.convert(h[0], np.float32)
                    else:
                        ref.arith(kind, h[0], h[1])
                    kw.update(cpu_ms=(time.perf_counter() - t0) * 1e3, cpu_kind="reference (u16 as int32)"
                              if host_in[0].dtype == np.uint16 else "reference")
                    kw["speedup_vs_cpu"] = kw["cpu_ms"] / ms
            except Exception:
                pass
            rec(name, ms, n, nbytes, **kw)

    def octagon4096():
        # the octagon compound SE (its cross passes, then one box for the trailing squares), 4096^2 u8 / u16
        from poutre2_gb300.se import Compound_NL_SE
        rng = np.random.default_rng(10)
        for dt, tdt in ((np.uint8, torch.uint8), (np.uint16, torch.uint16)):
            a = rng.integers(0, np.iinfo(dt).max, (4096, 4096), dtype=dt, endpoint=True)
            x = torch.from_numpy(a).to(dev)
            o = torch.empty_like(x)
            for size in (5, 10):
                ms = _time_ms(lambda: llm.Dilate(x, Compound_NL_SE.Octagon, size, o), flush, 15, 3)
                kw = {}
                try:
                    from oracle import ref
                    if ref.available() and dt == np.uint8:
                        t0 = time.perf_counter()
                        ref.erode_dilate_compound(a, "Octagon", size, True)
                        kw.update(cpu_ms=(time.perf_counter() - t0) * 1e3, cpu_kind="reference")
                        kw["speedup_vs_cpu"] = kw["cpu_ms"] / ms
                except Exception:
                    pass
                rec(f"octagon{size}_dilate_4096_{np.dtype(dt).name}", ms, a.size, 2 * a.nbytes, **kw)

    def geodesy3d():
        # binary h-maxima (h = 10) of a 128^3 u8 volume (white noise, Gaussian sigma 2, rescaled),
        # SECross3D: the iterated geodesic step of the volume route, poutre2 on one core beside it
        from scipy.ndimage import gaussian_filter
        rng = np.random.default_rng(12)
        v = gaussian_filter(rng.standard_normal((128, 128, 128)), 2.0, mode="reflect", truncate=4.0)
        f = np.rint((v - v.min()) / (v.max() - v.min()) * 255).astype(np.uint8)
        x = torch.from_numpy(f).to(dev)
        o = torch.empty_like(x)
        for se in ("SECross3D",):
            ms = _time_ms(lambda se=se: geo.h_maxima_binary(x, 10, Common_NL_SE[se], o, check=False), flush, 5, 2)
            kw = {"note": "includes the host reads of the change flag (every two brick launches)"}
            try:
                from oracle import ref
                if ref.available():
                    t0 = time.perf_counter()
                    ref.extrema("h_maxima", f, 10, se)
                    kw.update(cpu_ms=(time.perf_counter() - t0) * 1e3, cpu_kind="reference (h_maxima, compare not timed)")
                    kw["speedup_vs_cpu"] = kw["cpu_ms"] / ms
            except Exception:
                pass
            rec(f"h_maxima_binary_{se}_128cube_u8", ms, f.size, 2 * f.size, **kw)

    for fn in (cfg1, cfg2_4096, cfg2_leveling, cfg3, large, cfg4, cfg5, label2048, pixel4096, octagon4096, geodesy3d):
        if only is None or fn.__name__ in only:
            guard(fn)
    return res


def flush_l2(buf):
    """Evict L2 by reading a buffer twice its size (a read leaves clean lines, so the timed
    kernel pays no write-back of the flush)."""
    buf.max()


def run_gpu(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from poutre2_gb300 import _lib, geo
    from poutre2_gb300.se import Common_NL_SE
    _lib.load()
    geo.sync_checks = False

    f = workload_image(args.size)
    N = f.size
    dev = torch.device("cuda", local)
    x = torch.from_numpy(f).to(dev)
    out = torch.empty_like(x)
    flush = torch.ones(64 * 1024 * 1024, dtype=torch.int32, device=dev)  # 256 MB > L2 (129 MB)
    stream = torch.cuda.current_stream()

    def step():
        geo.h_maxima_binary(x, H_VALUE, Common_NL_SE.SESquare2D, out, check=False)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    _lib.call("pg_check_device", None)
    rounds = geo.last_reconstruction_rounds()

    # device-resident timed region: per-step events, L2 flushed between steps (untimed)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        time.sleep(0.5)  # let the sampler take its first readings before the timed steps
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush_l2(flush)
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    clocks = clk.summary()
    ms = [a.elapsed_time(b) for a, b in ev]
    t_step = max_over_ranks(sum(ms) / len(ms) / 1e3, ws, dev)
    _lib.call("pg_check_device", None)
    value = replica_value(N, ws, t_step)

    # parity of the timed output against the oracle and against poutre2 itself (outside the timed region)
    import oracle
    got = out.cpu().numpy()
    parity = bool(np.array_equal(got, oracle.h_maxima_binary(f, H_VALUE, "SESquare2D")))
    parity_ref = None
    try:
        from oracle import ref
        if ref.available():
            parity_ref = bool(np.array_equal(got, ref.h_maxima_binary(f, H_VALUE, "SESquare2D")))
    except Exception:
        parity_ref = None

    # end to end through the public API, every step's copies inside the timed region: pinned host input
    # -> device -> binary result -> pinned host.  (a) serial: one step at a time, L2 flushed before each;
    # (b) the reported figure: the steps alternate between two streams, so that one step's copies overlap
    # the other's kernel, as a serving loop runs them; its time per step is the loop's time / K.
    hin = torch.from_numpy(f).pin_memory()
    hout = torch.empty(f.shape, dtype=torch.uint8).pin_memory()
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        flush_l2(flush)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        xd = hin.to(dev, non_blocking=True)
        od = torch.empty_like(xd)
        geo.h_maxima_binary(xd, H_VALUE, Common_NL_SE.SESquare2D, od, check=False)
        hout.copy_(od, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append(a.elapsed_time(b))
    t_e2e_serial = max_over_ranks(sum(e2e_ms) / len(e2e_ms) / 1e3, ws, dev)

    streams = [torch.cuda.Stream(device=dev) for _ in range(2)]
    hins = [torch.from_numpy(f).pin_memory() for _ in range(2)]
    houts = [torch.zeros(f.shape, dtype=torch.uint8).pin_memory() for _ in range(2)]
    dins = [torch.empty(f.shape, dtype=torch.uint8, device=dev) for _ in range(2)]
    douts = [torch.empty_like(d) for d in dins]

    def e2e_step(i):
        k = i % 2
        with torch.cuda.stream(streams[k]):
            dins[k].copy_(hins[k], non_blocking=True)
            geo.h_maxima_binary(dins[k], H_VALUE, Common_NL_SE.SESquare2D, douts[k], check=False)
            houts[k].copy_(douts[k], non_blocking=True)

    for i in range(args.warmup):
        e2e_step(i)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for st in streams:
        st.wait_stream(stream)
    for i in range(args.steps):
        e2e_step(i)
    for st in streams:
        stream.wait_stream(st)
    b.record(stream)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(a.elapsed_time(b) / args.steps / 1e3, ws, dev)
    e2e_parity = all(np.array_equal(h.numpy(), got) for h in houts)

    peak, peak_kind = peaks()
    alg_bytes = 2 * N  # mask read + binary output written, per launch
    achieved = alg_bytes / t_step / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8", "data": "synthetic",
        "config": {"workload": workload_name(args.size), "parallelism": f"replicas x{ws}",
                   "l2": "flushed between timed steps (256 MB read, untimed)", "rounds": rounds},
        "parity_vs_oracle": parity, "parity_vs_reference": parity_ref,
        "e2e": {"value": replica_value(N, ws, t_e2e), "unit": UNIT, "h2d_bytes_per_step": int(N), "d2h_bytes_per_step": int(N),
                "ms_per_step": t_e2e * 1e3, "how": "K steps alternating over two streams (copies of one step overlap the "
                                                  "other's kernel), loop time / K; every step's H2D and D2H copies inside",
                "serial_ms_per_step": t_e2e_serial * 1e3, "serial_value": replica_value(N, ws, t_e2e_serial),
                "parity_of_copied_results": e2e_parity},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic_for(f"k_reconstruct_wl@hmaxima{args.size}"),
                     "peak_source": f"{peak_kind} hbm_gbs (burst)", "kernel": "k_reconstruct_wl<u8,dilate,8-conn>",
                     "algorithmic_bytes_per_launch": alg_bytes},
        "gpu_launches": args.steps,  # one persistent k_reconstruct_wl launch per step (plus one memset)
        "clocks": clocks,
    }
    if rank == 0:
        if not args.no_cpu:
            th = cpu_threads()
            v, kind, runs = cpu_hmaxima(f, budget_s=args.cpu_budget, threads=th)
            v1, _, runs1 = cpu_hmaxima(f, budget_s=min(args.cpu_budget, 5.0))
            line["cpu_baseline"] = {"value": v / 1e9, "unit": UNIT, "cores": th, "kind": kind, **host_cpu(),
                                    "sample": f"{runs} runs; each run: {th} host threads each run the full "
                                              f"{args.size}^2 workload on its own copy (poutre2 is single-threaded)",
                                    "single_thread_value": v1 / 1e9, "single_thread_runs": runs1,
                                    "build": f"g++ -O3 ({platform.machine()}; xsimd stand-in of fixed-width lane "
                                             f"loops, auto-vectorised by the compiler)"}
        if args.extra:
            only = set(args.only.split(",")) if args.only else None
            line["extra"] = extra_measurements(dev, flush, only, args.cfg5_batch)
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--extra", action="store_true", default=True, help="also measure the other workloads (default)")
    ap.add_argument("--no-extra", dest="extra", action="store_false")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--only", default="", help="comma-separated subset of the extra workloads (e.g. cfg3,cfg5)")
    ap.add_argument("--cfg5-batch", type=int, default=64, help="first dimension of the cfg5 tensor (64 = the workload; "
                                                              "smaller only for profiling captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
