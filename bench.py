"""Benchmark of the integer image pipeline on GB300.

Workload (one step): one 4096x4096 u8 image through the 3x3 Sobel magnitude
min(|gx|+|gy|, 255) with Boundary::MIRROR and the fused global u64 sum and u8
max of the result, plus one 4096x4096 uchar4 image through the RGBA->gray
point operator (77R + 150G + 29B) >> 8.  Steps rotate over NSETS resident
image pairs (NSETS x 117 MB, several times the 129 MB L2), so every step reads
its inputs from HBM.  The timed steps are replayed from CUDA graphs of up to
64 steps each.  Every step is independent of the others and its two operators
of each other, so a graph holds two chains on two streams, forked at its start
and joined at its end: the steps' Sobel launches in step order on one stream
(they share the library's reduction workspace) and their gray launches on the
other.  A step's gray may therefore run beside the next step's Sobel.

Metric: Gpixels/s = (Sobel pixels + gray pixels) per second, whole job.
`roofline` is for the dominant kernel (the one with the longer launch: Sobel at
2 algorithmic bytes per pixel or gray at 5); `kernels` lists both kernels'
achieved HBM bandwidth.
`e2e` drives the same step through the C ABI with host buffers
(hgb_image_write / kernels / hgb_image_read_async): pinned host -> device
copies of both inputs and device -> host reads of both outputs and the two
scalars every step, two steps in flight (one uploading while the other reads
back).

--impl reference times the reference's CPU path for the same step (the
oracle's restatement of the CPU back end, OpenMP over all host cores).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = H = 4096
PX_PER_STEP = 2 * W * H  # Sobel pixels + gray pixels
SOBEL_BYTES = 2 * W * H  # u8 in + u8 out (sum / max fused: 0 extra)
GRAY_BYTES = 5 * W * H  # uchar4 in + u8 out
NSETS = 16
# DRAM bytes (read + write) per launch from one ncu capture of each kernel on
# this workload (profiles/ holds the summary and the command); most of each
# kernel's output is still in L2 when the capture ends, so writes read low
NCU_TRAFFIC = {"sobel3_tma_kernel": 16845312 + 0, "gray_bulk_kernel": 67121152 + 1238016}
E2E_STEPS = 64  # end-to-end steps timed, independent of --steps
METRIC = "Gpixels/s (Sobel3x3 MIRROR + u64 sum + u8 max, and RGBA->gray, 4096x4096)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-extras", action="store_true", help="skip the other workloads' kernel timings")
    ap.add_argument("--only", default=None, choices=list(OTHER_SECTIONS),
                    help="time one of the other workloads alone (a short run, e.g. for a profiler) and exit")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def aggregate(elapsed_s: float, pixels: float, world: int):
    """Max time and summed pixels over ranks (identity for one process)."""
    if world <= 1:
        return elapsed_s, pixels
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([elapsed_s], dtype=torch.float64, device=dev)
    p = torch.tensor([pixels], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(t.item()), float(p.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------- CPU
def cpu_step_inputs(seed=0):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (H, W), dtype=np.uint8)
    rgba = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    return img, rgba


def cpu_step(O, img, rgba, nthreads):
    mag = O.sobel_mag(img, boundary=O.MIRROR, nthreads=nthreads)
    s = O.reduce_sum_u8(mag, nthreads=nthreads)
    m = O.reduce_max_u8(mag, nthreads=nthreads)
    g = O.rgba_to_gray(rgba, nthreads=nthreads)
    return mag, s, m, g


def cpu_time(seconds: float, nthreads: int):
    """Steps of the CPU path for about `seconds`; returns (px/s, steps)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    img, rgba = cpu_step_inputs(7)
    cpu_step(O, img, rgba, nthreads)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        cpu_step(O, img, rgba, nthreads)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return n * PX_PER_STEP / el, n, el


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    cores = os.cpu_count() or 1
    img, rgba = cpu_step_inputs(7)
    for _ in range(max(0, min(args.warmup, 2))):
        cpu_step(O, img, rgba, cores)
    steps = max(1, min(args.steps, 20))  # bounded sample of the same step
    t0 = time.perf_counter()
    for _ in range(steps):
        cpu_step(O, img, rgba, cores)
    el = time.perf_counter() - t0
    v = steps * PX_PER_STEP / el / 1e9
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Gpixels/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": el / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded uniform u8 / uchar4)",
        "config": {"workload": "sobel3x3_mirror_sum_max+rgba_gray_4096x4096", "width": W, "height": H},
        "cpu_baseline": {"value": v, "unit": "Gpixels/s", "cores": cores, "kind": "port",
                         "sample": f"{steps} full steps of the 4096x4096 pipeline (reference CPU back end restated,"
                                   f" OpenMP over rows)"},
        "e2e": {"value": v, "unit": "Gpixels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference CPU back end restated in C++/OpenMP: the reference is not a Python package (pip install"
                " finds no setup.py or pyproject.toml), its compiler needs Clang 10 and its CUDA runtime does not"
                " build on CUDA 13",
    }))


# --------------------------------------------------------------------- GPU
def run_gb300(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from hipacc_gb300 import _lib as L
    from hipacc_gb300 import api

    api.init(local)
    dev = torch.device("cuda", local)
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    imgs = [torch.randint(0, 256, (H, W), dtype=torch.uint8, device=dev, generator=g) for _ in range(NSETS)]
    rgbas = [torch.randint(0, 256, (H, W, 4), dtype=torch.uint8, device=dev, generator=g) for _ in range(NSETS)]
    mags = [torch.empty((H, W), dtype=torch.uint8, device=dev) for _ in range(NSETS)]
    grays = [torch.empty((H, W), dtype=torch.uint8, device=dev) for _ in range(NSETS)]
    sums = torch.zeros((NSETS,), dtype=torch.int64, device=dev)
    maxs = torch.zeros((NSETS,), dtype=torch.int32, device=dev)
    L.call("hgb_workspace_reserve", 64 << 20)

    def sobel(i, stream=None):
        api.sobel_mag(imgs[i], mags[i], boundary=api.MIRROR, sum_out=sums[i:i + 1], max_out=maxs[i:i + 1],
                      stream=stream)

    def gray(i, stream=None):
        api.gray(rgbas[i], grays[i], stream=stream)

    side = torch.cuda.Stream(device=dev)

    def steps(ks, stream=None):
        # steps ks as two chains forked from and joined back into `stream`:
        # every Sobel in step order on it, every gray on the side stream
        st = stream if stream is not None else torch.cuda.current_stream()
        fork = torch.cuda.Event()
        fork.record(st)
        side.wait_event(fork)
        for i in ks:
            sobel(i % NSETS, st)
        for i in ks:
            gray(i % NSETS, side)
        join = torch.cuda.Event()
        join.record(side)
        st.wait_event(join)

    # eager warm-up over every resident set
    steps(range(NSETS))
    torch.cuda.synchronize()

    s = torch.cuda.Stream(device=dev)

    def capture(fn, n, base=0):
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            fn(range(NSETS), s)  # warm on the capture stream
            torch.cuda.synchronize()
            with torch.cuda.graph(gr, stream=s):
                fn(range(base, base + n), s)
        torch.cuda.synchronize()
        return gr

    def per_kernel(fn):
        return lambda ks, st: [fn(i % NSETS, st) for i in ks]

    # the K timed steps: graphs of up to 64 steps, rotating over the resident sets
    g_timed = [capture(steps, min(64, args.steps - a), a) for a in range(0, args.steps, 64)]
    g_warm = capture(steps, max(3, args.warmup))
    g_sobel = capture(per_kernel(sobel), NSETS)
    g_gray = capture(per_kernel(gray), NSETS)

    # the clock sampler runs from before the warm-up to after the timed
    # region, so the GPU does not sit idle between the two
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.25)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    # warm-up: max(3, W) steps, then one replay of each timed graph so that
    # its first launch (which uploads it to the device) is not the timed one
    with torch.cuda.stream(s):
        g_warm.replay()
        for gr in g_timed:
            gr.replay()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s):
        e0.record(s)
        for gr in g_timed:
            gr.replay()
        e1.record(s)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    # per-kernel average launch duration, same stream, same rotation
    kern = {}
    for name, gr, nbytes in (("sobel3_tma_kernel", g_sobel, SOBEL_BYTES), ("gray_bulk_kernel", g_gray, GRAY_BYTES)):
        reps = max(4, args.steps // NSETS // 2)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s):
            gr.replay()
            a.record(s)
            for _ in range(reps):
                gr.replay()
            b.record(s)
        torch.cuda.synchronize()
        us = a.elapsed_time(b) * 1e3 / (reps * NSETS)
        kern[name] = {"us_per_launch": us, "algorithmic_bytes": nbytes, "achieved_gbs": nbytes / us / 1e3}
    clk = clocks.stop()
    elapsed = e0.elapsed_time(e1) / 1e3
    elapsed_max, px_total = aggregate(elapsed, args.steps * PX_PER_STEP, world)
    value = px_total / elapsed_max / 1e9

    # ---- end to end through the C ABI with host buffers
    e2e = run_e2e(args, L, dev, rank)
    e2e_max, e2e_px = aggregate(e2e["elapsed"], e2e["pixels"], world)

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1:
        cores = os.cpu_count() or 1
        pxs, n, el = cpu_time(args.cpu_seconds, cores)
        cpu = {"value": pxs / 1e9, "unit": "Gpixels/s", "cores": cores, "kind": "port",
               "sample": f"{n} full 4096x4096 steps in {el:.1f} s (reference CPU back end restated, OpenMP)"}

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    others = measure_other_configs(dev, peak) if (rank == 0 and not args.no_extras) else None
    dom_name = max(kern, key=lambda k: kern[k]["us_per_launch"])  # the kernel with the larger share of the step
    dom = kern[dom_name]
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gpixels/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_max / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded uniform u8 / uchar4)",
            "config": {"workload": "sobel3x3_mirror_sum_max+rgba_gray_4096x4096", "width": W, "height": H,
                       "images_per_step": "1 u8 + 1 uchar4", "pixels_per_step": PX_PER_STEP,
                       "resident_sets": NSETS, "l2": f"inputs larger than L2 ({NSETS} rotating sets, "
                                                     f"{NSETS * 117} MB)", "launch": "CUDA graph replay: graphs of up to 64 steps, each a Sobel chain and a gray chain on two streams",
                       "parallelism": f"replicas x{world}",
                       "warmup_detail": f"{max(3, args.warmup)} steps, then one untimed replay of each timed graph "
                                        f"({args.steps} steps) so that no timed launch is a graph's first"},
            "roofline": {"bound": "hbm", "achieved": dom["achieved_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": dom["achieved_gbs"] / peak, "traffic": NCU_TRAFFIC.get(dom_name), "kernel": dom_name,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s"},
            "kernels": kern,
            "other_configs": others,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_px / e2e_max / 1e9, "unit": "Gpixels/s", "h2d_bytes_per_step": e2e["h2d"],
                    "d2h_bytes_per_step": e2e["d2h"], "steps": e2e["steps"]},
            "gpu_launches": 2 * args.steps,
            "clocks": clk,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def graph_time_us(fn, n, stream, reps):
    """Average device time of fn(i) (i = 0..n-1, one launch each) replayed from
    a CUDA graph on `stream`, in microseconds per launch."""
    import torch

    with torch.cuda.stream(stream):
        for i in range(n):
            fn(i)
    torch.cuda.synchronize()
    gr = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gr, stream=stream):
        for i in range(n):
            fn(i)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        gr.replay()
        a.record(stream)
        for _ in range(reps):
            gr.replay()
        b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) * 1e3 / (reps * n)


def field(h, w, seed, dev):
    """Smooth 2-D sinusoid plus N(0, 0.05) noise clipped to [0, 1] (the
    precision workload's image), generated on the device."""
    import torch

    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    y = torch.arange(h, device=dev, dtype=torch.float32)[:, None]
    x = torch.arange(w, device=dev, dtype=torch.float32)[None, :]
    f = 0.5 + 0.25 * torch.sin(2 * np.pi * x / 512.0) * torch.cos(2 * np.pi * y / 384.0)
    f = f + 0.05 * torch.randn((h, w), device=dev, generator=g)
    return f.clamp_(0.0, 1.0)


def gauss_taps(k, sigma):
    ax = np.arange(-(k // 2), k // 2 + 1, dtype=np.float64)
    g = np.exp(-ax ** 2 / (2 * sigma * sigma))
    return (g / g.sum()).astype(np.float32)


OTHER_SECTIONS = ("integer", "gaussian", "precision", "pyramid", "diff", "histogram", "pipelines", "extras",
                  "pyramid_trace")


def measure_other_configs(dev, peak_gbs, only=None):
    """Device throughput of the other workloads (graph-replayed, inputs larger than L2).
    `only` restricts the run to one section with the fewest replays."""
    import torch

    from hipacc_gb300 import api

    s = torch.cuda.Stream(device=dev)
    res = {}
    q = 1 if only else 0  # replays shrink to one in a single-section run

    def want(sec):
        return only is None or only == sec

    if only == "integer":  # the headline step's two kernels alone, few launches (for a profiler)
        _integer(dev, peak_gbs, s, res)
    if only == "pyramid_trace":  # where the single launch spends its time (measurement only)
        _pyramid_trace(dev, s, res)
    if want("gaussian"):
        _gaussian(dev, peak_gbs, s, res, q)
    if want("precision"):
        _precision(dev, peak_gbs, s, res, q)
    if want("pyramid"):
        _pyramid(dev, peak_gbs, s, res, q)
    if want("diff"):
        _diff(dev, s, res, q)
    if want("histogram"):
        _histogram(dev, peak_gbs, s, res, q)
    if want("pipelines"):
        _pipelines(dev, peak_gbs, s, res, q)
    if want("extras"):
        _extras(dev, peak_gbs, s, res, q)
    return res


def _integer(dev, peak_gbs, s, res):
    import torch

    from hipacc_gb300 import api

    g = torch.Generator(device=dev)
    g.manual_seed(7)
    n = 4
    imgs = [torch.randint(0, 256, (H, W), dtype=torch.uint8, device=dev, generator=g) for _ in range(n)]
    rgbas = [torch.randint(0, 256, (H, W, 4), dtype=torch.uint8, device=dev, generator=g) for _ in range(n)]
    mags = [torch.empty_like(x) for x in imgs]
    grays = [torch.empty((H, W), dtype=torch.uint8, device=dev) for _ in range(n)]
    acc = torch.zeros((n, 2), dtype=torch.int64, device=dev)
    us = graph_time_us(lambda i: api.sobel_mag(imgs[i], mags[i], boundary=api.MIRROR, sum_out=acc[i, 0:1],
                                               max_out=acc[i, 1:2], stream=s), n, s, 2)
    res["sobel3_mirror_sum_max_4096"] = {"us_per_launch": us, "achieved_gbs": SOBEL_BYTES / us / 1e3,
                                         "frac_hbm": SOBEL_BYTES / us / 1e3 / peak_gbs}
    us = graph_time_us(lambda i: api.gray(rgbas[i], grays[i], stream=s), n, s, 2)
    res["rgba_gray_4096"] = {"us_per_launch": us, "achieved_gbs": GRAY_BYTES / us / 1e3,
                             "frac_hbm": GRAY_BYTES / us / 1e3 / peak_gbs}


def _extras(dev, peak_gbs, s, res, q):
    """The remaining operators of the path, each alone: standalone global reductions, resampling
    accessors, and the two adjoints.  Rotating inputs larger than L2."""
    import torch

    from hipacc_gb300 import api

    g = torch.Generator(device=dev)
    g.manual_seed(17)
    n, px = 8, 4096 * 4096
    reps = 1 if q else 10
    u8 = [torch.randint(0, 256, (4096, 4096), dtype=torch.uint8, device=dev, generator=g) for _ in range(n)]
    r8 = torch.zeros(n, dtype=torch.int64, device=dev)
    us = graph_time_us(lambda i: api.L.call("hgb_reduce", C.byref(api.view(u8[i])), None, api.SUM,
                                            C.c_void_p(r8[i:i + 1].data_ptr()), None, api._stream(s)), n, s, reps)
    res["reduce_sum_u8_u64_4096"] = {"us_per_launch": us, "gpix_s": px / us / 1e3, "achieved_gbs": px / us / 1e3,
                                     "frac_hbm": px / us / 1e3 / peak_gbs}
    del u8
    f32 = [torch.rand((4096, 4096), device=dev, generator=g) for _ in range(n)]
    rf = torch.zeros(n, dtype=torch.float64, device=dev)
    us = graph_time_us(lambda i: api.L.call("hgb_reduce", C.byref(api.view(f32[i])), None, api.SUM,
                                            C.c_void_p(rf[i:i + 1].data_ptr()), None, api._stream(s)), n, s, reps)
    res["reduce_sum_f32_kahan_4096"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                        "achieved_gbs": 4 * px / us / 1e3, "frac_hbm": 4 * px / us / 1e3 / peak_gbs}
    # resampling accessors: 2048^2 -> 4096^2 (4 bytes read per output / 4 plus 4 written)
    src = [torch.rand((2048, 2048), device=dev, generator=g) for _ in range(n)]
    dst = [torch.empty((4096, 4096), device=dev) for _ in range(n)]
    for mode in ("nn", "lf", "b5", "cf", "l3"):
        us = graph_time_us(lambda i: api.resample(src[i], dst[i], mode, stream=s), n, s, reps)
        b = 4 * px + 4 * px // 4
        res[f"resample_{mode}_2048_to_4096"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                                "achieved_gbs": b / us / 1e3, "frac_hbm": b / us / 1e3 / peak_gbs}
    del src, dst
    # adjoints: 7x7 SUM local operator (grad_in + grad_mask) and 9x9 bilateral (grad_in + grad_sigma)
    gout = [torch.randn((4096, 4096), device=dev, generator=g) for _ in range(n)]
    m7 = np.random.default_rng(3).normal(0, 0.1, (7, 7)).astype(np.float32)
    us = graph_time_us(lambda i: api.local_op_adjoint(gout[i], m7, api.CLAMP, inp=f32[i], stream=s), n, s, reps)
    res["local_op_adjoint7_f32_4096"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                         "achieved_gbs": 12 * px / us / 1e3, "frac_hbm": 12 * px / us / 1e3 / peak_gbs}
    ax = np.arange(-4, 5, dtype=np.float64)
    sm9 = np.exp(-(ax[None, :] ** 2 + ax[:, None] ** 2) / (2 * 4.0)).astype(np.float32)
    us = graph_time_us(lambda i: api.bilateral_adjoint(f32[i], gout[i], sm9, 0.15, api.CLAMP, stream=s), n, s,
                       max(1, reps // 5))
    res["bilateral_adjoint9_f32_4096"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                          "exp_per_s": 2 * 81 * px / us * 1e6}
    del gout, f32


def _pipelines(dev, peak_gbs, s, res, q):
    import torch

    from hipacc_gb300 import api

    # the Harris corner and Unsharp sample programs at the samples' 4032 x 3024,
    # fused against the reference's nine / five launches; 8 rotating images
    # (Harris 195 MB, Unsharp 780 MB of inputs and outputs, larger than L2)
    w, h, n = 4032, 3024, 8
    g = torch.Generator(device=dev)
    g.manual_seed(13)
    px = w * h
    ins = [torch.randint(0, 256, (h, w), dtype=torch.uint8, device=dev, generator=g) for _ in range(n)]
    outs = [torch.empty_like(x) for x in ins]
    for mode, name in ((0, "fused_1launch"), (1, "reference_9launches")):
        us = graph_time_us(lambda i: api.harris(ins[i], outs[i], boundary=api.CLAMP, mode=mode, stream=s), n, s,
                           1 if q else 10)
        res[f"harris3_{w}x{h}_{name}"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                          "achieved_gbs": 2 * px / us / 1e3, "frac_hbm": 2 * px / us / 1e3 / peak_gbs}
    del ins, outs
    ins = [torch.randint(0, 256, (h, w, 4), dtype=torch.uint8, device=dev, generator=g) for _ in range(n)]
    outs = [torch.empty_like(x) for x in ins]
    for mode, name in ((0, "fused_1launch"), (1, "reference_5launches")):
        us = graph_time_us(lambda i: api.unsharp(ins[i], outs[i], boundary=api.CLAMP, mode=mode, stream=s), n, s,
                           1 if q else 10)
        res[f"unsharp3_{w}x{h}_{name}"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                           "achieved_gbs": 8 * px / us / 1e3, "frac_hbm": 8 * px / us / 1e3 / peak_gbs}
    del ins, outs


def _histogram(dev, peak_gbs, s, res, q):
    import torch

    from hipacc_gb300 import api

    # binned data of the histogram binning function, 256 bins, 4096x4096 u8 and f32
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    px = 4096 * 4096
    for name, make, es in (("u8", lambda: torch.randint(0, 256, (4096, 4096), dtype=torch.uint8, device=dev,
                                                        generator=g), 1),
                           ("f32", lambda: torch.rand((4096, 4096), device=dev, generator=g) * 255.0, 4)):
        ins = [make() for _ in range(8)]
        bins = [torch.empty(256, dtype=torch.int32, device=dev) for _ in range(8)]
        us = graph_time_us(lambda i: api.histogram(ins[i], 256, bins=bins[i], stream=s), 8, s, 2 if q else 20)
        res[f"histogram256_{name}_4096"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                            "achieved_gbs": es * px / us / 1e3,
                                            "frac_hbm": es * px / us / 1e3 / peak_gbs}
        del ins


def _gaussian(dev, peak_gbs, s, res, q):
    import torch

    from hipacc_gb300 import api

    # 5x5 sigma=1 Gaussian, FP32 1024x1024, CLAMP: batches of 64 distinct images per launch
    ax = np.arange(-2, 3, dtype=np.float64)
    m5 = np.exp(-(ax[None, :] ** 2 + ax[:, None] ** 2) / 2.0)
    m5 = (m5 / m5.sum()).astype(np.float32)
    nb = 4
    ins = [torch.rand((64, 1024, 1024), device=dev) for _ in range(nb)]
    outs = [torch.empty_like(x) for x in ins]
    us = graph_time_us(lambda i: api.local_op(ins[i % nb], outs[i % nb], mask=m5, boundary=api.CLAMP, stream=s), nb,
                       s, 1 if q else 10)
    px = 64 * 1024 * 1024
    res["gaussian5x5_f32_1024_clamp_b64"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                             "achieved_gbs": 8 * px / us / 1e3, "frac_hbm": 8 * px / us / 1e3 / peak_gbs}
    del ins, outs
    # the Gaussian-blur sample's own storage: u8 in and out, (uchar)(sum + 0.5f)
    ins = [torch.randint(0, 256, (64, 1024, 1024), dtype=torch.uint8, device=dev) for _ in range(nb)]
    outs = [torch.empty_like(x) for x in ins]
    us = graph_time_us(lambda i: api.local_op(ins[i % nb], outs[i % nb], mask=m5, boundary=api.CLAMP, stream=s), nb,
                       s, 1 if q else 10)
    res["gaussian5x5_u8_1024_clamp_b64"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                            "achieved_gbs": 2 * px / us / 1e3, "frac_hbm": 2 * px / us / 1e3 / peak_gbs}
    # the same launch with the tile configuration chosen by the autotuner (first, untimed call)
    api.autotune(True)
    try:
        api.local_op(ins[0], outs[0], mask=m5, boundary=api.CLAMP, stream=s)
        s.synchronize()
        us = graph_time_us(lambda i: api.local_op(ins[i % nb], outs[i % nb], mask=m5, boundary=api.CLAMP, stream=s),
                           nb, s, 1 if q else 10)
    finally:
        api.autotune(False)
    res["gaussian5x5_u8_1024_clamp_b64_autotuned"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                                      "achieved_gbs": 2 * px / us / 1e3,
                                                      "frac_hbm": 2 * px / us / 1e3 / peak_gbs}
    del ins, outs


def _precision(dev, peak_gbs, s, res, q):
    import torch

    from hipacc_gb300 import api

    # precision: separable 9x9 sigma=2 and 13x13 bilateral on 8192x8192, REPEAT
    img32 = [field(8192, 8192, 20 + i, dev) for i in range(2)]
    taps = gauss_taps(9, 2.0)
    ax = np.arange(-6, 7, dtype=np.float64)
    sm = np.exp(-(ax[None, :] ** 2 + ax[:, None] ** 2) / (2 * 9.0)).astype(np.float32)
    px = 8192 * 8192
    for name, dt in (("f32", torch.float32), ("bf16", torch.bfloat16), ("f16", torch.float16)):
        ins = [x.to(dt) for x in img32]
        outs = [torch.empty_like(x) for x in ins]
        es = ins[0].element_size()
        us = graph_time_us(lambda i: api.separable(ins[i % 2], outs[i % 2], taps, taps, boundary=api.REPEAT,
                                                   stream=s), 2, s, 1 if q else 10)
        res[f"separable9_{name}_8192_repeat"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                                 "achieved_gbs": 2 * es * px / us / 1e3,
                                                 "frac_hbm": 2 * es * px / us / 1e3 / peak_gbs}
        us = graph_time_us(lambda i: api.bilateral(ins[i % 2], outs[i % 2], sm, 0.1, boundary=api.REPEAT, stream=s),
                           2, s, 2)
        res[f"bilateral13_{name}_8192_repeat"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                                  "exp_per_s": 169 * px / us * 1e6}
        if dt != torch.float32:
            us = graph_time_us(lambda i: api.bilateral(ins[i % 2], outs[i % 2], sm, 0.1, boundary=api.REPEAT,
                                                       fast_weights=True, stream=s), 2, s, 2)
            res[f"bilateral13_{name}_halfweights_8192_repeat"] = {"us_per_launch": us, "gpix_s": px / us / 1e3,
                                                                  "exp_per_s": 169 * px / us * 1e6}
        del ins, outs
    res["precision_error_vs_fp64"] = _precision_errors(img32[0], taps, sm)
    del img32


def _err(got, ref):
    """max-abs and max-relative (max-abs / max |ref|) error of got against an FP64 reference."""
    got = np.asarray(got, np.float64)
    d = float(np.max(np.abs(got - ref)))
    return {"max_abs": d, "max_rel": d / max(float(np.max(np.abs(ref))), 1e-300)}


def _precision_errors(img, taps, sm):
    """Error of each storage type against the FP64 oracle, outside the timed region: the same kernels on
    the 512 x 512 corner crop of the benchmarked field (as a whole image, so both borders and interior
    count), against FP64 on the FP32 crop (input rounding of BF16 / FP16 storage included)."""
    import torch

    from hipacc_gb300 import api

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    crop = img[:512, :512].contiguous()
    c64 = crop.double().cpu().numpy()
    out = {}
    for b, bname in ((api.REPEAT, "repeat"), (api.CONSTANT, "constant0.5")):
        ref_sep = O.separable(c64, taps.astype(np.float64), taps.astype(np.float64), boundary=b, const=0.5)
        ref_bil = O.bilateral(c64, sm.astype(np.float64), 0.1, boundary=b, const=0.5)
        for name, dt in (("f32", torch.float32), ("bf16", torch.bfloat16), ("f16", torch.float16)):
            x = crop.to(dt)
            y = api.separable(x, None, taps, taps, boundary=b, const=0.5)
            out[f"separable9_{name}_{bname}"] = _err(y.double().cpu().numpy(), ref_sep)
            y = api.bilateral(x, None, sm, 0.1, boundary=b, const=0.5)
            out[f"bilateral13_{name}_{bname}"] = _err(y.double().cpu().numpy(), ref_bil)
            if dt != torch.float32:
                y = api.bilateral(x, None, sm, 0.1, boundary=b, const=0.5, fast_weights=True)
                out[f"bilateral13_{name}_halfweights_{bname}"] = _err(y.double().cpu().numpy(), ref_bil)
    torch.cuda.synchronize()
    return out


def _pyramid_batch(dev):
    """The pyramid workload: 64 FP32 images, w and h uniform in [257, 4096], 8 levels, MIRROR."""
    import torch

    from hipacc_gb300 import api

    rng = np.random.default_rng(4096)
    ws_ = rng.integers(257, 4097, 64)
    hs_ = rng.integers(257, 4097, 64)
    levels = 8
    b1 = np.array([1, 4, 6, 4, 1], np.float64) / 16.0
    plan = api.PyramidPlan(ws_, hs_, levels, np.outer(b1, b1).astype(np.float32), api.MIRROR)
    for i in range(64):
        plan.gauss(i, 0).copy_(torch.rand((int(hs_[i]), int(ws_[i])), device=dev))
    return plan, ws_, hs_, levels, b1


def _pyramid_trace(dev, s, res):
    """Per-CTA records of the three single-launch forms (hgb_pyramid_plan_trace), each at the tile
    configuration the autotuner picks for the single launch, beside the per-level launches: where
    the time goes (tile claims, waits on the previous level, tiles, the tail of the launch)."""
    import tempfile

    import torch

    from hipacc_gb300 import api

    plan, ws_, hs_, levels, b1 = _pyramid_batch(dev)
    api.autotune(True)
    plan.decompose(0, stream=s)
    plan.decompose(1, stream=s)
    s.synchronize()
    api.autotune(False)
    tuned = os.path.join(tempfile.gettempdir(), f"hgb_pyr_trace_{os.getpid()}.json")
    api.L.call("hgb_autotune_save", tuned.encode())
    table = json.load(open(tuned))
    key = [k for k in table if k.startswith("pyramid:m0:")][0]
    cfg = int(table[key][0]) % 4
    res["pyramid_trace_config"] = {"key": key, "autotuned": table[key], "tile_config": cfg}
    res["per_level_7launches_us"] = graph_time_us(lambda i: plan.decompose(1, stream=s), 1, s, 5)
    cap = 400000
    buf = torch.zeros(8 * cap, dtype=torch.int64, device=dev)
    for single, name in ((0, "persistent_claims"), (1, "one_cta_per_tile"), (2, "cooperative_static_level0")):
        json.dump({key: [single * 4 + cfg, 0.0]}, open(tuned, "w"))
        api.L.call("hgb_autotune_load", tuned.encode())
        us = graph_time_us(lambda i: plan.decompose(0, stream=s), 1, s, 5)
        buf.zero_()
        plan.trace(buf)
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(s)
        plan.decompose(0, stream=s)
        stop.record(s)
        s.synchronize()
        plan.trace(None)
        r = buf.view(-1, 8).cpu().numpy()
        r = r[r[:, 1] > 0]
        t0, t1, c0, c1 = r[:, 0], r[:, 1], r[:, 2], r[:, 3]
        life = (c1 - c0).astype(np.float64)
        span = float(t1.max() - t0.min())
        ends = np.sort(t1 - t0.min()) / 1e3
        tiles = (r[:, 7] & 0xffffffff).astype(np.int64)
        polled = (r[:, 7] >> 32).astype(np.int64)
        res[f"pyramid_trace_{name}"] = {
            "us_untraced": us, "us_traced": start.elapsed_time(stop) * 1e3, "ctas": int(len(r)),
            "span_us": span / 1e3, "tiles": int(tiles.sum()), "waits_that_polled": int(polled.sum()),
            "share_of_cta_cycles": {"claim": float(r[:, 4].sum() / life.sum()),
                                    "level_wait": float(r[:, 5].sum() / life.sum()),
                                    "tiles": float(r[:, 6].sum() / life.sum())},
            "cta_end_us_quantiles": {"first": float(ends[0]), "p10": float(np.quantile(ends, 0.1)),
                                     "p50": float(np.quantile(ends, 0.5)), "p90": float(np.quantile(ends, 0.9)),
                                     "last": float(ends[-1])},
        }
    os.remove(tuned)
    plan.close()


def _pyramid(dev, peak_gbs, s, res, q):
    import torch

    from hipacc_gb300 import api

    # batching: 64 FP32 images, w and h uniform in [257, 4096], 8-level Laplacian pyramid, MIRROR
    plan, ws_, hs_, levels, b1 = _pyramid_batch(dev)
    base_px = float(np.sum(ws_.astype(np.int64) * hs_))
    alg = 0.0
    for i in range(64):
        w, h = int(ws_[i]), int(hs_[i])
        for _ in range(levels - 1):
            alg += 8.0 * w * h + 4.0 * (w // 2) * (h // 2)  # read G_l, write L_l, write G_{l+1}
            w, h = w // 2, h // 2
    # the fused launch forms pick their tile configuration with the autotuner (first, untimed call)
    api.autotune(True)
    for mode, name in ((0, "persistent_1launch"), (1, "per_level_7launches"), (2, "per_image_per_level_1344launches")):
        us = graph_time_us(lambda i: plan.decompose(mode, stream=s), 1, s, 1 if q else (3 if mode < 2 else 2))
        res[f"pyramid8_64img_{name}"] = {"us_per_batch": us, "gpix_s": base_px / us / 1e3,
                                         "achieved_gbs": alg / us / 1e3, "frac_hbm": alg / us / 1e3 / peak_gbs}
    api.autotune(False)
    import tempfile

    tuned = os.path.join(tempfile.gettempdir(), f"hgb_pyramid_autotune_{os.getpid()}.json")
    try:
        api.L.call("hgb_autotune_save", tuned.encode())
        res["pyramid8_autotuned_choices"] = {k: v for k, v in json.load(open(tuned)).items() if k.startswith("pyramid")}
        os.remove(tuned)
    except (OSError, ValueError):
        pass
    # error of the persistent form's levels against the FP64 oracle, outside the timed region: the
    # smallest image of the batch, every level
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    plan.decompose(0, stream=s)
    torch.cuda.synchronize()
    i = int(np.argmin(ws_.astype(np.int64) * hs_))
    g64, l64 = O.pyramid_decompose(plan.gauss(i, 0).double().cpu().numpy(), levels, b1[:, None] * b1[None, :],
                                   O.MIRROR)
    err = {"image": f"{int(ws_[i])}x{int(hs_[i])}"}
    for l in range(levels):
        err[f"gauss{l}"] = _err(plan.gauss(i, l).double().cpu().numpy(), g64[l])
        if l + 1 < levels:
            err[f"lap{l}"] = _err(plan.lap(i, l).double().cpu().numpy(), l64[l])
    res["pyramid8_error_vs_fp64"] = err
    plan.close()


def _diff(dev, s, res, q):
    import torch

    from hipacc_gb300 import api

    # differentiation: 16 x 2048^2, learnable 7x7 mask + 9x9 bilateral (sigma_d = 2) with learnable sigma_r
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    x = torch.rand((16, 2048, 2048), device=dev, generator=g)
    ax = np.arange(-3, 4, dtype=np.float64)
    g15 = np.exp(-(ax[None, :] ** 2 + ax[:, None] ** 2) / (2 * 1.5 * 1.5))
    g15 = (g15 / g15.sum()).astype(np.float32)
    t = torch.empty_like(x)
    api.local_op(x, t, mask=g15, boundary=api.CLAMP)
    mask = (torch.randn((7, 7), device=dev, generator=g) * 0.02).contiguous()
    sigma = torch.tensor([0.15], device=dev)
    ax9 = np.arange(-4, 5, dtype=np.float64)
    sm9 = np.exp(-(ax9[None, :] ** 2 + ax9[:, None] ** 2) / (2 * 4.0)).astype(np.float32)
    px = 16 * 2048 * 2048
    for mode, name in ((0, "fused_3launches"), (1, "unfused_per_image")):
        us = graph_time_us(lambda i: api.conv_bilateral_mse(x, t, mask, sigma, sm9, api.CLAMP, mode, stream=s), 1, s,
                           1 if q else 3)
        res[f"conv7_bilateral9_mse_fwd_adj_16x2048_{name}"] = {"us_per_batch": us, "gpix_s": px / us / 1e3}
    # error against the FP64 oracle's forward + hand adjoint (pinned to FP64 central differences by the
    # tests), outside the timed region: image 0 of the batch as its own launch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    loss, gx, gm, gs = api.conv_bilateral_mse(x[0:1], t[0:1], mask, sigma, sm9, api.CLAMP, 0, stream=s)
    torch.cuda.synchronize()
    l0, dx0, dm0, ds0 = O.c5_grad(x[0].cpu().numpy(), t[0].cpu().numpy(), mask.double().cpu().numpy(),
                                  sm9.astype(np.float64), 0.15, O.CLAMP)
    rel = lambda a, b: float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))
    res["conv7_bilateral9_mse_error_vs_fp64"] = {
        "image": "2048x2048 (image 0 of the batch), CLAMP",
        "loss_rel": abs(float(loss.item()) - l0) / abs(l0),
        "grad_x_rel_l2": rel(gx[0].double().cpu().numpy(), dx0),
        "grad_mask_rel_l2": rel(gm.double().cpu().numpy(), dm0),
        "grad_sigma_rel": abs(float(gs.item()) - ds0) / abs(ds0)}
    del x, t


def run_e2e(args, L, dev, rank):
    """Host buffers in, host results out, every step through the C ABI.

    Each step uploads its two input images from pinned host memory
    (hgb_image_write), runs the Sobel (+ fused sum / max) and gray kernels and
    queues the read-back of both output images and both scalars.  Steps
    alternate between two device image sets on two streams, so one step's
    read-back and the next step's upload overlap on the link; the kernels of
    consecutive steps are ordered by an event (they share the library's
    reduction workspace).  The timed region ends when every read-back landed.
    """
    import torch

    lib = L.load()
    rng = np.random.default_rng(99 + rank)
    n_e2e = E2E_STEPS
    h_img = torch.from_numpy(rng.integers(0, 256, (H, W), dtype=np.uint8)).pin_memory()
    h_rgba = torch.from_numpy(rng.integers(0, 256, (H, W, 4), dtype=np.uint8)).pin_memory()
    nset = 2
    h_mag = [torch.empty((H, W), dtype=torch.uint8).pin_memory() for _ in range(nset)]
    h_gray = [torch.empty((H, W), dtype=torch.uint8).pin_memory() for _ in range(nset)]
    h_scalars = [torch.empty(2, dtype=torch.int64).pin_memory() for _ in range(nset)]
    sets = []
    for _ in range(nset):
        imgs, views = {}, {}
        for name, dt in (("img", L.U8), ("rgba", L.U8X4), ("mag", L.U8), ("gray", L.U8)):
            p = C.c_void_p()
            L.check(lib.hgb_image_create(dt, W, H, 256, None, C.byref(p)))
            v = L.View()
            L.check(lib.hgb_image_get_view(p, C.byref(v)))
            imgs[name], views[name] = p, v
        sets.append((imgs, views, torch.zeros(2, dtype=torch.int64, device=dev)))
    streams = [torch.cuda.Stream(device=dev) for _ in range(nset)]
    done = [torch.cuda.Event() for _ in range(nset)]
    mx = np.array([-1, 0, 1, -2, 0, 2, -1, 0, 1], np.int32)
    my = np.array([-1, -2, -1, 0, 0, 0, 1, 2, 1], np.int32)

    def one(k):
        j = k % nset
        imgs, views, scal = sets[j]
        st = streams[j]
        sp = C.c_void_p(st.cuda_stream)
        L.check(lib.hgb_image_write(imgs["img"], C.c_void_p(h_img.data_ptr()), sp))
        L.check(lib.hgb_image_write(imgs["rgba"], C.c_void_p(h_rgba.data_ptr()), sp))
        if k > 0:
            st.wait_event(done[(k - 1) % nset])  # kernels in step order
        L.check(lib.hgb_sobel_mag(C.byref(views["img"]), C.byref(views["mag"]), mx.ctypes.data_as(C.c_void_p),
                                  my.ctypes.data_as(C.c_void_p), 3, L.MIRROR, 0, C.c_void_p(scal.data_ptr()),
                                  C.c_void_p(scal.data_ptr() + 8), sp))
        L.check(lib.hgb_point_gray(C.byref(views["rgba"]), C.byref(views["gray"]), 77, 150, 29, 8, sp))
        done[j].record(st)
        L.check(lib.hgb_image_read_async(imgs["mag"], C.c_void_p(h_mag[j].data_ptr()), sp))
        L.check(lib.hgb_image_read_async(imgs["gray"], C.c_void_p(h_gray[j].data_ptr()), sp))
        with torch.cuda.stream(st):
            h_scalars[j].copy_(scal, non_blocking=True)

    for k in range(4):
        one(k)
    torch.cuda.synchronize()
    # the warm-up read-backs must be right: gray against numpy, the fused sum / max against the read-back image
    rgba = h_rgba.numpy().astype(np.uint32)
    ref_gray = ((77 * rgba[..., 0] + 150 * rgba[..., 1] + 29 * rgba[..., 2]) >> 8).astype(np.uint8)
    mag = h_mag[1].numpy()
    if not (np.array_equal(h_gray[1].numpy(), ref_gray) and int(h_scalars[1][0]) == int(mag.sum(dtype=np.uint64))
            and int(h_scalars[1][1]) == int(mag.max())):
        raise RuntimeError("end-to-end read-back does not match")
    t0 = time.perf_counter()
    for k in range(n_e2e):
        one(k)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    for imgs, _, _ in sets:
        for p in imgs.values():
            lib.hgb_image_destroy(p)
    return {"elapsed": el, "pixels": n_e2e * PX_PER_STEP, "steps": n_e2e, "h2d": W * H * 5,
            "d2h": W * H * 2 + 16}


def run_only(args):
    import torch

    from hipacc_gb300 import api

    api.init(0)
    dev = torch.device("cuda", 0)
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        peak = 6800.0
    print(json.dumps({"only": args.only, "timings": measure_other_configs(dev, peak, only=args.only)}))


def main():
    args = parse()
    if args.only:
        run_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
