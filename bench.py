"""Benchmark of the GB300 RDP path.

One step = one frame of the workload: a textured, depth-tested 320x240
RGBA5551 + Z16 frame, 2-cycle, 10,000 perspective-correct triangles (log-normal
area, median 48 px), RGBA16 32x32 textures with random wrap/mirror/clamp,
bilinear filtering, random combiner inputs, fog blender, Z compare + update,
coverage AA and magic-square dither, generated from seed 0.

value  : reference-equivalent render passes per second with every input already
         resident in HBM (the frame's passes replayed as a CUDA graph; CUDA events
         on the processor's stream; L2 flushed between timed iterations).
e2e    : the same metric through the C ABI with host buffers: command words in
         host memory are parsed, packed and copied H2D, the frame renders, and the
         written framebuffer is copied D2H into the caller's RDRAM, every step.
roofline: the rasteriser kernel (k_raster) -- algorithmic framebuffer bytes of the
         touched tiles / its CUDA-event duration, against the measured HBM copy peak.
cpu_baseline: the CPU oracle (a scalar restatement of the reference's algorithm)
         timed on this host on a bounded sample of the same frames.

--impl reference times the reference algorithm on the host CPU (the oracle; the
reference's own Vulkan/Angrylion build is not available) with the same metric.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "parallel-rdp_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "bit-exact RDP passes/s, Mpix/s on 1 GB300: batched+learned vs plain; p99 ms"
UNIT = "passes/s"
WORKLOAD = ("textured depth-tested frame: 320x240 RGBA5551 + Z16, 2-cycle, 10,000 perspective-correct triangles "
            "(log-normal area, median 48 px), RGBA16 32x32 LoadTile textures, bilinear, random combiner, fog blender, "
            "Z compare+update, coverage AA, magic-square dither, seed 0")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="env://")
    return dist, dist.get_rank(), ws, int(os.environ.get("LOCAL_RANK", "0"))


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def _frame():
    from rdp_gb300 import cmdgen
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=0)
    words, rdram, prims = cmdgen.generate_stream(p)
    return words, rdram, prims, p


def _fb_bytes_per_pixel(p):
    return 4 if p.fb_format == 1 else 2


def _l2_flusher(device):
    import torch
    buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda:%d" % device)

    def flush():
        buf.random_(0, 255)
        torch.cuda.synchronize(device)
    return flush


def _cpu_baseline(words, rdram, min_seconds=10.0, max_frames=30):
    """Oracle on this host, one thread, whole frames until >= min_seconds."""
    from oracle import Oracle
    frames, t0 = 0, time.perf_counter()
    passes = frags = 0
    while True:
        o = Oracle(8 << 20)
        o.write_rdram(rdram)
        o.enqueue(words)
        frags += o.fragments()
        frames += 1
        o.close()
        el = time.perf_counter() - t0
        if el >= min_seconds or frames >= max_frames:
            break
    return frames, el, frags


def _reference_passes(words, rdram):
    """Reference-equivalent pass count of one frame (host-side need_flush emulation)."""
    from rdp_gb300 import CommandProcessor
    rd = rdram.copy()
    with CommandProcessor(rd) as cp:
        cp.enqueue_command(words)
        cp.idle()
        s = cp.stats()
    return s


def run_ours(args):
    dist, rank, world, local = _dist()
    import torch
    torch.cuda.set_device(local)
    from rdp_gb300 import CommandProcessor

    words, rdram, prims, params = _frame()
    base = _reference_passes(words, rdram)
    passes_per_frame = base["reference_passes"]
    frags_per_frame = base["fragments"]
    tiles_per_frame = base["touched_tiles"]
    flush = _l2_flusher(local)

    # ---------------- value: device-resident graph replay
    rd = rdram.copy()
    cp = CommandProcessor(rd, device=local)
    graph = cp.capture(words)
    for _ in range(args.warmup):
        flush()
        graph.replay(1)
    clocks = ClockSampler(local)
    launches0 = cp.stats()["kernel_launches"]
    _barrier(dist)
    clocks.start()
    step_ms, raster_ms = [], []
    for _ in range(args.steps):
        flush()
        step_ms.append(graph.replay(1))
        raster_ms.append(graph.last_raster_ms())
    clock_info = clocks.stop()
    _barrier(dist)
    launches = cp.stats()["kernel_launches"] - launches0
    t_value = _max_over_ranks(dist, sum(step_ms) / 1e3)
    total_passes = _sum_over_ranks(dist, passes_per_frame * args.steps)
    total_frags = _sum_over_ranks(dist, frags_per_frame * args.steps)
    value = total_passes / t_value
    graph.close()

    # ---------------- e2e: C ABI with host buffers
    for _ in range(args.warmup):
        cp.enqueue_command(words)
        cp.wait_for_timeline(cp.signal_timeline())
    s0 = cp.stats()
    _barrier(dist)
    e2e_s = 0.0
    for _ in range(args.steps):
        flush()
        t0 = time.perf_counter()
        cp.enqueue_command(words)
        cp.wait_for_timeline(cp.signal_timeline())
        e2e_s += time.perf_counter() - t0
    s1 = cp.stats()
    _barrier(dist)
    e2e_t = _max_over_ranks(dist, e2e_s)
    e2e_value = total_passes / e2e_t
    h2d = (s1["staging_bytes"] - s0["staging_bytes"]) / args.steps
    d2h = params.width * params.height * (_fb_bytes_per_pixel(params) + 2)  # colour + depth images copied back
    cp.close()

    # ---------------- roofline of the rasteriser
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    # Per touched 8x8 tile: colour (2 B) + hidden (1 B) + depth (2 B) + hidden (1 B) per pixel, read and written.
    bytes_per_tile = 64 * (2 + 1 + 2 + 1) * 2
    raster_launch_ms = statistics.mean(raster_ms) / max(1, base["passes"])
    algo_bytes = tiles_per_frame * bytes_per_tile / max(1, base["passes"])
    achieved = algo_bytes / (raster_launch_ms / 1e3) / 1e9 if raster_launch_ms > 0 else 0.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "k_raster_traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            traffic = None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_value * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (seeded RDP command words)",
        "config": {"workload": WORKLOAD, "frames_per_step": 1, "primitives_per_frame": prims,
                   "reference_passes_per_frame": passes_per_frame, "fragments_per_frame": frags_per_frame,
                   "parallelism": "replicas" if world > 1 else "single", "l2": "flushed between timed iterations"},
        "mpix_per_s": total_frags / t_value / 1e6,
        "frames_per_s": world * args.steps / t_value,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "mpix_per_s": total_frags / e2e_t / 1e6},
        "gpu_launches": int(launches),
        "roofline": {"kernel": "k_raster", "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": peak_src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": raster_launch_ms},
        "clocks": clock_info,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        frames, el, frags = _cpu_baseline(words, rdram)
        line["cpu_baseline"] = {"value": passes_per_frame * frames / el, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "%d whole frames of the workload through the CPU oracle, one thread" % frames,
                                "mpix_per_s": frags / el / 1e6}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args):
    """The reference algorithm on the host CPU (the oracle), same metric and config."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    words, rdram, prims, params = _frame()
    from oracle import Oracle
    ncores = os.cpu_count() or 1

    def one_frame():
        o = Oracle(8 << 20)
        o.write_rdram(rdram)
        o.enqueue(words)
        f = o.fragments()
        o.close()
        return f

    # Reference-equivalent passes per frame, counted with the same host emulation as our arm.
    try:
        passes_per_frame = _reference_passes(words, rdram)["reference_passes"]
    except Exception:
        passes_per_frame = (prims + 255) // 256
    for _ in range(args.warmup):
        one_frame()
    t0 = time.perf_counter()
    frags = 0
    for _ in range(args.steps):
        frags += one_frame()
    el = time.perf_counter() - t0
    value = passes_per_frame * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded RDP command words)",
        "config": {"workload": WORKLOAD, "frames_per_step": 1, "primitives_per_frame": prims},
        "mpix_per_s": frags / el / 1e6,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "one whole frame per step through the CPU oracle (scalar restatement of the "
                                   "reference algorithm; the reference's Vulkan build needs a graphics stack); "
                                   "%d host cores available, 1 used" % ncores},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
