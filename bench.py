"""Benchmark of the GB300 RDP path.

Default workload (--workload batched): the batched-instances configuration --
64 independent emulator instances, each with its own 8 MiB RDRAM and 4 KiB TMEM,
resolutions drawn from 320x240 / 640x240 / 640x480, primitive counts log-uniform
in 500-50,000 per frame, the mixed RGBA8888 primitive mix (40% textured
triangles, 30% copy-mode TextureRectangles, 20% CI8 + TLUT triangles, 10%
FillRects; alpha compare, LOD/detail and Z on half the primitives), per-instance
seeds 0-63.  One step = one frame of every instance (one sync point).

value  : reference-equivalent render passes per second (the reference's pass rule,
         counted by the host emulation of its need_flush) of the BATCHED path with the
         LEARNED tile order (the cost model trains online on the first sync points) and
         every input resident in HBM: the sync point's rounds replayed as a CUDA graph;
         CUDA events on the batch's stream; L2 flushed between iterations.  The same
         replay in plain tile order is reported beside it (tile_order.static).
plain  : the same frames through the plain single-instance path, one processor and
         one CUDA graph per instance, run one after another.
e2e    : the batched path through the C ABI with host buffers: every instance's
         command words are parsed, packed and copied H2D, all instances render, and
         written framebuffers are copied D2H into each caller's RDRAM, every step.  The
         steps run as a frame server's loop: step s+1 is parsed and submitted while step
         s renders, then step s's results are waited for (e2e.serial_value: one step at
         a time).
roofline: the dominant kernel (k_shade): bytes of its output (the 8 B shaded record per
         pixel of every shaded (primitive, 8x8 tile) pair -- the reference writes a 10 B
         record -- plus the 8 B pair entry), per launch, over its CUDA-event duration,
         against the HBM copy peak; `traffic` scales the DRAM bytes per pair of a scoped
         one-kernel ncu capture.  roofline.int_alu: the integer-op roofline that binds this
         integer fixed-point work -- the reference algorithm's integer ops per step, counted
         on the CPU oracle per stage (oracle/op_table.json, made by oracle/make_op_table.py),
         over the measured time, against the integer issue peak (SMs x 4 sub-partitions x 32
         lanes x the sampled SM clock).  roofline.step_hbm: the step's algorithmic bytes
         (command words, the touched tiles' framebuffer loads and stores, texture sources)
         over the step time, against the HBM peak.
cpu_baseline: the CPU oracle (a scalar restatement of the reference's algorithm)
         over the instances on all host cores, on a bounded sample (>= 10 s).

--workload plain / textured / mixed measures one processor on the plain 2,000-triangle frame, the
textured depth-tested frame (10,000 triangles) or the mixed 640x480 sequence (16 frames x 50,000
primitives, VI scanout of each frame in the end-to-end loop) instead.  --impl reference times the reference algorithm on the
host CPU (the oracle, all host threads; the reference's own Vulkan/Angrylion build
is not available) on the same workload and metric.
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
BATCH_INSTANCES = 64
BATCH_WORKLOAD = ("batched instances: 64 emulator instances (8 MiB RDRAM + 4 KiB TMEM each), resolutions from "
                  "320x240/640x240/640x480, 500-50,000 primitives per frame (log-uniform), mixed RGBA8888 primitive "
                  "mix (textured / copy TexRect / CI8+TLUT / FillRect, alpha compare, LOD, Z on half), seeds 0-63, "
                  "one frame per instance per step")
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
        """Starts sampling every 50 ms and returns once the first sample is in (at most ~1 s),
        so that the samples cover the timed region that follows."""
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        deadline = time.time() + 1.0
        while time.time() < deadline and self.proc.poll() is None and os.path.getsize(self.path) == 0:
            time.sleep(0.01)

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


# Single-processor workloads: (generator config, description, op-table key, VI scanout per frame).
SINGLE = {
    "plain": (0, "plain single frame: 320x240 RGBA5551, 1-cycle, a FillRect clear then 2,000 Gouraud triangles "
                 "(vertices uniform over the screen, log-normal area median 64 px sigma 1.5, RGBA shade uniform), SHADE "
                 "combiner, pass-through blender, dither off, seed 0", "plain", False),
    "textured": (1, WORKLOAD, "textured", False),
    "mixed": (2, "mixed 640x480 RGBA8888 sequence: 16 frames x 50,000 primitives (40 % textured triangles, 30 % "
                 "copy-mode TextureRectangles, 20 % CI8 + 256-entry TLUT triangles, 10 % FillRects; alpha compare, "
                 "LOD / detail tiles and Z on half), VI scanout of every frame (AA filter, divot, dither filter, "
                 "interlaced 640x480), seed 0", "mixed16", True),
}


def _frame(workload="textured"):
    """Command words of one step of a single-processor workload (every frame of it), the initial
    RDRAM, the primitive count, the generator parameters and each frame's first word."""
    from rdp_gb300 import cmdgen
    p = cmdgen.default_params(SINGLE[workload][0], seed=0)
    words, rdram, prims, offsets = cmdgen.generate_frames(p)
    return words, rdram, prims, p, offsets


def _fb_bytes_per_pixel(p):
    return 4 if p.fb_format == 1 else 2


def _l2_flusher(device):
    import torch
    buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda:%d" % device)

    def flush():
        buf.random_(0, 255)
        torch.cuda.synchronize(device)
    return flush


def _cpu_frames(words, rdram, offsets, min_seconds=10.0, max_rounds=30):
    """The CPU oracle on one thread over the workload's frames in order (the step repeated from a
    fresh RDRAM when it is short) until >= min_seconds.  Returns (frames, reference passes,
    fragments, seconds)."""
    from oracle import Oracle
    nf = len(offsets) - 1
    frames = passes = frags = 0
    t0 = time.perf_counter()
    for _ in range(max_rounds):
        o = Oracle(8 << 20)
        o.write_rdram(rdram)
        for f in range(nf):
            o.enqueue(words[offsets[f]:offsets[f + 1]])
            frames += 1
            if time.perf_counter() - t0 >= min_seconds:
                break
        passes += o.reference_passes()
        frags += o.fragments()
        o.close()
        if time.perf_counter() - t0 >= min_seconds:
            break
    return frames, passes, frags, time.perf_counter() - t0


def _mixed_vi_regs(frame):
    """VI registers of the mixed sequence's scanout: the 640x480 RGBA8888 colour image, AA filter
    with resampling, divot, dither filter, interlaced (field = frame parity)."""
    from rdp_gb300 import VIRegister, cmdgen

    def start(a, b):
        return ((a & 0x3ff) << 16) | (b & 0x3ff)

    return {VIRegister.Control: 3 | (1 << 4) | (1 << 16) | (1 << 6), VIRegister.Origin: cmdgen.color_addr(),
            VIRegister.Width: 640, VIRegister.VSync: 525, VIRegister.VStart: start(34, 34 + 480),
            VIRegister.HStart: start(108, 108 + 640), VIRegister.XScale: 1024, VIRegister.YScale: 2048,
            VIRegister.VCurrentLine: frame & 1}


def _peaks():
    """HBM peak (GB/s) and its source: the measured copy bandwidth when the driver has written
    MEASURED_PEAKS.json, else the recipe's fallback figure."""
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        peaks = {}
    if "hbm_gbs" in peaks:
        return float(peaks["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _sm_count(device):
    import torch
    return torch.cuda.get_device_properties(device).multi_processor_count


def _int_alu_roofline(workload, step_ms, shade_ms, sm_count, sm_mhz):
    """Integer-op roofline of the step and of the shading kernel.  Ops are the reference
    algorithm's integer / logic ops per step, counted per stage on the CPU oracle (data in
    oracle/op_table.json); the peak is the integer issue rate, one 32-lane instruction per SM
    sub-partition per cycle at the SM clock sampled during the timed region."""
    try:
        table = json.load(open(os.path.join(ROOT, "oracle", "op_table.json")))["workloads"][workload]
    except (OSError, ValueError, KeyError):
        return None
    mhz = sm_mhz or 2070.0
    peak = sm_count * 4 * 32 * mhz * 1e6 / 1e12  # Tops/s
    step_ops, shade_ops = table["ops_total"], table["ops_shading_stages"]
    step_t = step_ops / (step_ms / 1e3) / 1e12
    shade_t = shade_ops / (shade_ms / 1e3) / 1e12 if shade_ms > 0 else 0.0
    return {"bound": "int_alu", "unit": "Tops/s", "peak": peak,
            "peak_source": "spec: %d SMs x 4 sub-partitions x 32 lanes x %.0f MHz (sampled SM clock)" % (sm_count, mhz),
            "ops_per_step": step_ops, "achieved": step_t, "frac": step_t / peak,
            "k_shade": {"ops_per_step": shade_ops, "achieved": shade_t, "frac": shade_t / peak},
            "ops_source": "oracle/op_table.json (%s): per-stage integer ops of the reference algorithm" % workload}


def _step_hbm_roofline(cmd_bytes, touched_tiles, fb_bytes_per_tile, uploads, step_ms, peak, peak_src):
    """The step's algorithmic bytes: command words, each touched 8x8 tile's framebuffer loaded and
    stored once (colour + hidden bytes, and 16-bit depth + hidden for images with a depth
    buffer), and at most one 4 KiB TMEM image of texture source per upload."""
    algo = cmd_bytes + touched_tiles * fb_bytes_per_tile + uploads * 4096
    achieved = algo / (step_ms / 1e3) / 1e9
    return {"bound": "hbm", "unit": "GB/s", "algorithmic_bytes_per_step": algo, "achieved": achieved, "peak": peak,
            "peak_source": peak_src, "frac": achieved / peak}


def _shade_traffic_per_pair():
    """DRAM bytes per shaded pair of the shading kernel, from the scoped ncu capture summarised in
    profiles/k_shade_traffic.json (one kernel, a few launches, the 16-instance case)."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "k_shade_traffic.json"))).get("dram_bytes_per_pair")
    except (OSError, ValueError):
        return None


def _reference_passes(words, rdram):
    """Reference-equivalent pass count of one frame (host-side need_flush emulation)."""
    from rdp_gb300 import CommandProcessor
    rd = rdram.copy()
    with CommandProcessor(rd) as cp:
        cp.enqueue_command(words)
        cp.idle()
        s = cp.stats()
    return s


def run_ours_single(args):
    """One processor on a single-processor workload (plain frame, textured frame or the mixed
    16-frame sequence with VI): the whole step replayed from one CUDA graph with inputs resident
    (value), and the same through the C ABI with host buffers (e2e; the mixed sequence also scans
    every frame out)."""
    dist, rank, world, local = _dist()
    import torch
    torch.cuda.set_device(local)
    from rdp_gb300 import CommandProcessor

    workload_text, op_key, with_vi = SINGLE[args.workload][1:]
    words, rdram, prims, params, offsets = _frame(args.workload)
    frames_per_step = len(offsets) - 1
    base = _reference_passes(words, rdram)
    passes_per_frame = base["reference_passes"]
    frags_per_frame = base["fragments"]
    tiles_per_frame = base["touched_tiles"]
    flush = _l2_flusher(local)

    # ---------------- value: device-resident graph replay
    rd = rdram.copy()
    cp = CommandProcessor(rd, device=local)
    from rdp_gb300 import get_shade_variant
    for _ in range(16):  # the autotuner times the shading-kernel variants on the first frames
        if get_shade_variant(local) >= 0:
            break
        cp.enqueue_command(words)
        cp.idle()
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
        raster_ms.append(graph.last_shade_ms())
    clock_info = clocks.stop()
    _barrier(dist)
    launches = cp.stats()["kernel_launches"] - launches0
    graph_shade_launches = graph.shade_launches
    t_value = _max_over_ranks(dist, sum(step_ms) / 1e3)
    total_passes = _sum_over_ranks(dist, passes_per_frame * args.steps)
    total_frags = _sum_over_ranks(dist, frags_per_frame * args.steps)
    value = total_passes / t_value
    graph.close()

    # ---------------- e2e: C ABI with host buffers (every frame enqueued, signalled and waited for;
    # the mixed sequence also scanned out after each frame)
    vi_opts = None
    if with_vi:
        from rdp_gb300 import ScanoutOptions
        vi_opts = ScanoutOptions(blend_previous_frame=1, upscale_deinterlacing=0)

    def e2e_step():
        out = 0
        for f in range(frames_per_step):
            cp.enqueue_command(words[offsets[f]:offsets[f + 1]])
            if with_vi:
                for r, v in _mixed_vi_regs(f).items():
                    cp.set_vi_register(r, v)
                img = cp.scanout_sync(vi_opts)
                out += img.nbytes if img is not None else 0
            else:
                cp.wait_for_timeline(cp.signal_timeline())
        return out

    for _ in range(args.warmup):
        e2e_step()
    s0 = cp.stats()
    _barrier(dist)
    e2e_s, vi_bytes = 0.0, 0
    for _ in range(args.steps):
        flush()
        t0 = time.perf_counter()
        vi_bytes = e2e_step()
        e2e_s += time.perf_counter() - t0
    s1 = cp.stats()
    _barrier(dist)
    e2e_t = _max_over_ranks(dist, e2e_s)
    e2e_value = total_passes / e2e_t
    h2d = (s1["staging_bytes"] - s0["staging_bytes"]) / args.steps
    # colour + depth images written back each frame, plus the scanned-out images
    d2h = frames_per_step * params.width * params.height * (_fb_bytes_per_pixel(params) + 2) + vi_bytes
    cp.close()

    # ---------------- roofline of the rasteriser
    hbm_peak, peak_src = _peaks()
    bytes_per_pair = 64 * 8 + 8  # the 8-byte shaded record per pixel + the 8-byte pair entry
    shade_launches = max(1, graph_shade_launches)
    raster_launch_ms = statistics.mean(raster_ms) / shade_launches
    algo_bytes = base["tile_instances"] * bytes_per_pair / shade_launches
    achieved = algo_bytes / (raster_launch_ms / 1e3) / 1e9 if raster_launch_ms > 0 else 0.0
    # The scoped capture's DRAM bytes per pair were measured on the batched workload; this frame is
    # not captured, so its traffic is not reported.
    traffic = None
    step_ms_mean = t_value * 1e3 / args.steps
    int_alu = _int_alu_roofline(op_key, step_ms_mean, statistics.mean(raster_ms), _sm_count(local),
                                clock_info.get("sm_mhz"))
    # Colour + hidden bytes, and (textured, mixed) Z16 + hidden, loaded and stored per touched tile.
    cbytes = _fb_bytes_per_pixel(params) + (2 if params.fb_format == 1 else 1)
    zbytes = 3 if args.workload != "plain" else 0
    step_hbm = _step_hbm_roofline(len(words) * 4, base["touched_tiles"], 64 * 2 * (cbytes + zbytes),
                                  base["tmem_uploads"], step_ms_mean, hbm_peak, peak_src)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_value * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (seeded RDP command words)",
        "config": {"workload": workload_text, "frames_per_step": frames_per_step, "primitives_per_step": prims,
                   "reference_passes_per_step": passes_per_frame, "fragments_per_step": frags_per_frame,
                   "parallelism": "replicas" if world > 1 else "single", "l2": "flushed between timed iterations",
                   "e2e_vi_scanout": with_vi},
        "mpix_per_s": total_frags / t_value / 1e6,
        "frames_per_s": world * args.steps * frames_per_step / t_value,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "mpix_per_s": total_frags / e2e_t / 1e6},
        "gpu_launches": int(launches),
        "roofline": {"kernel": "k_shade", "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": peak_src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": raster_launch_ms,
                     "int_alu": int_alu, "step_hbm": step_hbm},
        "clocks": clock_info,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        done, passes, frags, el = _cpu_frames(words, rdram, offsets)
        line["cpu_baseline"] = {"value": passes / el, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "%d frames of the workload in order through the CPU oracle, one thread "
                                          "(>= 10 s)" % done, "mpix_per_s": frags / el / 1e6}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_reference_single(args):
    """The reference algorithm on the host CPU (the oracle), same workload, metric and unit: each
    step renders the workload's frames in order on one thread, bounded to a sample of frames
    (the mixed sequence: two frames per step, continuing where the last step stopped)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    workload_text = SINGLE[args.workload][1]
    words, rdram, prims, params, offsets = _frame(args.workload)
    from oracle import Oracle
    ncores = os.cpu_count() or 1
    nf = len(offsets) - 1
    per_step = nf if nf <= 2 else 2
    state = {"o": None, "next": 0}

    def step():
        passes = frags = 0
        for _ in range(per_step):
            if state["o"] is None or state["next"] == nf:
                if state["o"] is not None:
                    state["o"].close()
                state["o"] = Oracle(8 << 20)
                state["o"].write_rdram(rdram)
                state["next"] = 0
            o, f = state["o"], state["next"]
            p0, g0 = o.reference_passes(), o.fragments()
            o.enqueue(words[offsets[f]:offsets[f + 1]])
            passes += o.reference_passes() - p0
            frags += o.fragments() - g0
            state["next"] = f + 1
        return passes, frags

    for _ in range(args.warmup):
        step()
    passes = frags = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        p, f = step()
        passes += p
        frags += f
    el = time.perf_counter() - t0
    value = passes / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded RDP command words)",
        "config": {"workload": workload_text, "frames_per_step": per_step, "primitives_per_step": prims * per_step // nf},
        "mpix_per_s": frags / el / 1e6,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "%d frame(s) per step in order through the CPU oracle (scalar restatement of the "
                                   "reference algorithm; the reference's Vulkan build needs a graphics stack); "
                                   "%d host cores available, 1 used" % (per_step, ncores)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ============================================================================ batched instances
def _batched_streams(n):
    from rdp_gb300 import cmdgen
    out = []
    for i in range(n):
        p = cmdgen.batched_instance_params(i)
        words, rdram, prims = cmdgen.generate_stream(p)
        out.append((words, rdram, prims, p))
    return out


def _oracle_instances(streams, min_seconds=None, threads=None):
    """Renders instances through the CPU oracle on `threads` host threads (ctypes drops the
    GIL, so the threads run in parallel).  With min_seconds, stops starting new instances
    once that much time has passed.  Returns (instances done, passes, fragments, seconds)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import Oracle
    threads = threads or os.cpu_count() or 1
    stop = threading.Event()
    t0 = time.perf_counter()

    def one(item):
        words, rdram = item[0], item[1]
        if stop.is_set():
            return None
        o = Oracle(8 << 20)
        o.write_rdram(rdram)
        o.enqueue(words)
        r = (o.reference_passes(), o.fragments())
        o.close()
        if min_seconds is not None and time.perf_counter() - t0 >= min_seconds:
            stop.set()
        return r

    with ThreadPoolExecutor(max_workers=threads) as ex:
        results = list(ex.map(one, streams))
    el = time.perf_counter() - t0
    done = [r for r in results if r is not None]
    return len(done), sum(r[0] for r in done), sum(r[1] for r in done), el, threads


def _run_batch_step(b, insts, streams):
    # Command words of every instance parsed on host threads, then one submission.
    values = b.enqueue_many(insts, [st[0] for st in streams])
    b.submit()
    for cp, v in zip(insts, values):
        cp.wait_for_timeline(v)


def run_ours_batched(args):
    dist, rank, world, local = _dist()
    import torch
    torch.cuda.set_device(local)
    from rdp_gb300 import Batch, CommandProcessor

    streams = _batched_streams(args.instances)
    flush = _l2_flusher(local)
    prims_per_step = sum(st[2] for st in streams)

    # ---------------- batched processors; the first frame gives the per-step unit counts
    b = Batch(device=local)
    insts = [b.add_instance(st[1].copy()) for st in streams]
    s0 = [cp.stats() for cp in insts]
    _run_batch_step(b, insts, streams)
    s1 = [cp.stats() for cp in insts]
    b.idle()  # grows the pair scratch to what the sync point needed
    from rdp_gb300 import get_shade_order, get_shade_variant
    for _ in range(12):  # the autotuner times the shading-kernel variants on the first sync points
        if get_shade_variant(local) >= 0:
            break
        _run_batch_step(b, insts, streams)
        b.idle()
    passes_per_step = sum(x["reference_passes"] - y["reference_passes"] for x, y in zip(s1, s0))
    frags_per_step = sum(x["fragments"] - y["fragments"] for x, y in zip(s1, s0))
    pairs_per_step = sum(x["tile_instances"] - y["tile_instances"] for x, y in zip(s1, s0))
    tiles_per_step = sum(x["touched_tiles"] - y["touched_tiles"] for x, y in zip(s1, s0))
    uploads_per_step = sum(x["tmem_uploads"] - y["tmem_uploads"] for x, y in zip(s1, s0))

    # ---------------- learned tile order: the cost model trains online on the first sync points
    b.set_schedule(learned_order=True, train=True, learning_rate=3e-3)
    for _ in range(args.train_steps):
        _run_batch_step(b, insts, streams)
        b.idle()
    model_loss = b.get_model()[1]
    b.set_schedule(learned_order=True, train=False)

    def timed_graph(tag):
        graph = b.capture([st[0] for st in streams])
        for _ in range(args.warmup):
            flush()
            graph.replay(1)
        clocks = ClockSampler(local)
        _barrier(dist)
        clocks.start()
        step_ms, shade_ms, blend_ms = [], [], []
        for _ in range(args.steps):
            flush()
            step_ms.append(graph.replay(1))
            shade_ms.append(graph.last_shade_ms())
            blend_ms.append(graph.last_blend_ms())
        clock_info = clocks.stop()
        _barrier(dist)
        out = dict(step_ms=step_ms, shade_ms=shade_ms, blend_ms=blend_ms, clocks=clock_info,
                   launches=graph.kernels * args.steps, shade_launches=graph.shade_launches)
        graph.close()
        return out

    # ---------------- value: device-resident graph replay of the whole sync point (learned order)
    rl = timed_graph("learned")
    step_ms, shade_ms, clock_info = rl["step_ms"], rl["shade_ms"], rl["clocks"]
    launches, shade_launches = rl["launches"], rl["shade_launches"]
    t_value = _max_over_ranks(dist, sum(step_ms) / 1e3)
    total_passes = _sum_over_ranks(dist, passes_per_step * args.steps)
    total_frags = _sum_over_ranks(dist, frags_per_step * args.steps)
    value = total_passes / t_value
    # The same sync point in plain tile order (the fallback the learned order is compared with).
    b.set_schedule(learned_order=False, train=False)
    rs = timed_graph("static")
    t_static = _max_over_ranks(dist, sum(rs["step_ms"]) / 1e3)
    b.set_schedule(learned_order=True, train=False)

    # ---------------- e2e: C ABI with host buffers, all instances per step
    for _ in range(args.warmup):
        _run_batch_step(b, insts, streams)
    # One step at a time (L2 flushed before each): parse, submit, wait for every result.
    e2e_serial_s = 0.0
    for _ in range(args.steps):
        flush()
        t0 = time.perf_counter()
        _run_batch_step(b, insts, streams)
        e2e_serial_s += time.perf_counter() - t0
    # The frame loop of a frame server: step s+1's command words are parsed and submitted while
    # step s renders, then step s's results are waited for (its framebuffers are back in the
    # instances' host memory).  No L2 flush: each step stages ~200 MB of command data, more
    # than L2 holds.
    def frame_loop(steps):
        pending = None
        for _ in range(steps):
            values = b.enqueue_many(insts, [st[0] for st in streams])
            b.submit()
            if pending is not None:
                for cp, v in zip(insts, pending):
                    cp.wait_for_timeline(v)
            pending = values
        for cp, v in zip(insts, pending):
            cp.wait_for_timeline(v)

    frame_loop(args.warmup)  # the staging ring grows to the depth of the pipelined loop
    bs0 = b.stats()
    _barrier(dist)
    t0 = time.perf_counter()
    frame_loop(args.steps)
    e2e_s = time.perf_counter() - t0
    bs1 = b.stats()
    _barrier(dist)
    e2e_t = _max_over_ranks(dist, e2e_s)
    e2e_value = total_passes / e2e_t
    e2e_serial_value = total_passes / _max_over_ranks(dist, e2e_serial_s)
    h2d = (bs1["staging_bytes"] - bs0["staging_bytes"]) / args.steps
    d2h = sum(st[3].width * st[3].height * (4 + 2) for st in streams)  # colour + depth images copied back
    rounds_per_step = (bs1["rounds"] - bs0["rounds"]) / args.steps
    b_model = b.get_model()[0]
    b.close()

    # ---------------- plain: one processor + graph per instance, one after another
    plain_ms = 0.0
    per_instance_ms = []
    for st in streams:
        cp = CommandProcessor(st[1].copy(), device=local)
        g = cp.capture(st[0])
        for _ in range(1):
            flush()
            g.replay(1)
        ms = 0.0
        for _ in range(args.steps):
            flush()
            ms += g.replay(1)
        plain_ms += ms
        per_instance_ms.append(ms / args.steps)
        g.close()
        cp.close()
    t_plain = _max_over_ranks(dist, plain_ms / 1e3)
    plain_value = total_passes / t_plain
    # Where the plain path's time goes: the smallest instances' graph time is mostly the fixed cost
    # of a kernel chain; the rest grows with the work.
    order = sorted(range(len(streams)), key=lambda i: streams[i][2])
    small = [per_instance_ms[i] for i in order[:8]]
    plain_breakdown = {"instance_ms_min": min(per_instance_ms), "instance_ms_median": statistics.median(per_instance_ms),
                       "instance_ms_max": max(per_instance_ms),
                       "fixed_ms_per_instance_estimate": statistics.median(small),
                       "largest_instance_ms": per_instance_ms[order[-1]],
                       "largest_instance_primitives": int(streams[order[-1]][2])}

    # ---------------- serving: 256 instances, Poisson arrivals, continuous batching
    serving = None
    if not args.no_serving:
        serving = _serving(args, local, model=b_model)

    # ---------------- roofline of the dominant kernel
    hbm_peak, peak_src = _peaks()
    bytes_per_pair = 64 * 8 + 8  # the 8-byte shaded record per pixel + the 8-byte pair entry
    shade_launch_ms = statistics.mean(shade_ms) / max(1, shade_launches)
    algo_bytes = pairs_per_step * bytes_per_pair / max(1, shade_launches)
    achieved = algo_bytes / (shade_launch_ms / 1e3) / 1e9 if shade_launch_ms > 0 else 0.0
    per_pair = _shade_traffic_per_pair()
    traffic = per_pair * pairs_per_step / max(1, shade_launches) if per_pair else None
    step_ms_mean = t_value * 1e3 / args.steps
    int_alu = _int_alu_roofline("batched64", step_ms_mean, statistics.mean(shade_ms), _sm_count(local),
                                clock_info.get("sm_mhz")) if args.instances == BATCH_INSTANCES else None
    # RGBA8888 colour (4 B) + 2 hidden bytes and Z16 (2 B) + hidden (1 B) per pixel, loaded and stored.
    step_hbm = _step_hbm_roofline(sum(len(st[0]) for st in streams) * 4, tiles_per_step, 64 * 2 * (6 + 3),
                                  uploads_per_step, step_ms_mean, hbm_peak, peak_src)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_value * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (seeded RDP command words)",
        "config": {"workload": BATCH_WORKLOAD, "instances": args.instances, "primitives_per_step": prims_per_step,
                   "reference_passes_per_step": passes_per_step, "fragments_per_step": frags_per_step,
                   "tile_instances_per_step": pairs_per_step, "rounds_per_step": rounds_per_step,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between timed iterations", "tile_order": "learned (longest predicted first)",
                   "shade_variant": get_shade_variant(local), "shade_order": get_shade_order(local)},
        "mpix_per_s": total_frags / t_value / 1e6,
        "frames_per_s": world * args.steps * args.instances / t_value,
        "plain": {"value": plain_value, "unit": UNIT, "ms_per_step": t_plain * 1e3 / args.steps,
                  "mpix_per_s": total_frags / t_plain / 1e6, "breakdown": plain_breakdown},
        "batched_over_plain": value / plain_value,
        "tile_order": {"learned": {"ms_per_step": t_value * 1e3 / args.steps,
                                   "blend_ms_per_step": statistics.mean(rl["blend_ms"])},
                       "static": {"value": total_passes / t_static, "ms_per_step": t_static * 1e3 / args.steps,
                                  "blend_ms_per_step": statistics.mean(rs["blend_ms"])},
                       "model_train_steps": args.train_steps, "model_mse": model_loss},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "mpix_per_s": total_frags / e2e_t / 1e6, "loop": "pipelined frame loop (step s+1 submitted before "
                "waiting for step s), no L2 flush: ~200 MB staged per step", "serial_value": e2e_serial_value},
        "serving": serving,
        "gpu_launches": int(launches),
        "roofline": {"kernel": "k_shade", "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": peak_src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": shade_launch_ms,
                     "launches_per_step": shade_launches,
                     "share_of_step": statistics.mean(shade_ms) / statistics.mean(step_ms),
                     "int_alu": int_alu, "step_hbm": step_hbm},
        "clocks": clock_info,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n, passes, frags, el, threads = _oracle_instances(streams, min_seconds=10.0)
        line["cpu_baseline"] = {"value": passes / el, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d of the %d instances' frames through the CPU oracle, instances spread "
                                          "over %d host threads" % (n, len(streams), threads),
                                "mpix_per_s": frags / el / 1e6}
        # The serving configuration's 1 % output sample, checked against the oracle (untimed).
        if serving and serving.get("parity_sample"):
            serving["parity_sample"] = _check_serving_parity(serving["parity_sample"], threads)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def _serving(args, device, model=None):
    """The serving configuration: 256 instances with the batched workload's distribution of
    resolutions and primitive counts submit frames as a Poisson process; requests are admitted by
    HBM footprint; the learned tile order is on.  Runs the arrival rate of the configuration
    (20,000 frames/s aggregate, over a short window) and a rate the GPU can sustain."""
    from rdp_gb300 import Batch
    from rdp_gb300.serving import latency_summary, poisson_trace
    streams = _batched_streams(args.serve_instances)
    frames = [st[0] for st in streams]
    b = Batch(device=device)
    if model is not None:
        b.set_model(model)
    b.set_schedule(learned_order=True, train=False)
    insts = [b.add_instance(st[1].copy()) for st in streams]
    for cp, w in zip(insts, frames):  # warm-up: every instance renders once, buffers settle
        cp.enqueue_command(w)
    b.idle()
    for cp, w in zip(insts, frames):
        cp.enqueue_command(w)
    t0 = time.perf_counter()
    b.idle()
    renders = [2] * len(insts)  # frames each instance has rendered (for the parity sample)
    all_requests = []
    capacity_fps = len(insts) / (time.perf_counter() - t0)
    out = {"instances": len(insts), "hbm_budget_gb": args.serve_budget_gb, "capacity_fps_estimate": capacity_fps}
    # The configured rate first; the sustainable rate is 80 % of what the serving loop delivered
    # under that overload (its own capacity with Poisson-sized batches, below the full-batch one).
    for tag, dur in (("configured_rate", args.serve_window), ("sustainable", 1.0)):
        rate = 20000.0 if tag == "configured_rate" else 0.8 * out["configured_rate"]["throughput_fps"]
        trace = poisson_trace(len(insts), rate, dur, frames, seed=42)
        res, st = b.serve(insts, trace, hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)))
        for t in trace:
            renders[t[0]] += 1
            all_requests.append(t[0])
        lat = latency_summary(res["latency_s"])
        span = float(res["done_s"].max() - min(t[2] for t in trace)) if len(trace) else 0.0
        lat.update({"rate_fps": rate, "window_s": dur, "throughput_fps": len(trace) / span if span > 0 else 0.0,
                    "submits": st["submits"], "max_in_flight": st["max_in_flight"],
                    "max_footprint_gb": st["max_footprint"] / (1 << 30)})
        out[tag] = lat
    # Latency floor: the largest instance's frame alone on an idle GPU (one request, nothing else
    # in flight), end to end through the serving loop.
    big = max(range(len(streams)), key=lambda i: streams[i][2])
    floor = []
    for k in range(5):
        res, _ = b.serve(insts, [(big, frames[big], 0.0)], hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)))
        floor.append(float(res["latency_s"][0]) * 1e3)
        renders[big] += 1
    out["latency_floor"] = {"instance": big, "primitives": int(streams[big][2]),
                            "resolution": "%dx%d" % (streams[big][3].width, streams[big][3].height),
                            "alone_ms_min": min(floor), "alone_ms_median": statistics.median(floor)}
    out["parity_sample"] = _serving_parity_sample(insts, all_requests, renders)
    b.close()
    return out


def _serving_parity_sample(insts, requests, renders, fraction=0.01, seed=7):
    """The serving configuration's output check, first half: a seeded 1 % sample of the served
    requests; for each sampled request's instance, the digests of its RDRAM and hidden RDRAM after
    the run and how many times it rendered its frame.  The CPU-baseline leg renders those instances'
    frames as many times through the oracle and compares (_check_serving_parity)."""
    import hashlib
    if not requests:
        return {"requests_sampled": 0, "instances": {}}
    rng = np.random.default_rng(seed)
    k = max(1, int(round(fraction * len(requests))))
    picks = sorted(int(i) for i in rng.choice(len(requests), size=min(k, len(requests)), replace=False))
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()  # noqa: E731
    inst = {}
    for i in sorted({requests[j] for j in picks}):
        inst[i] = {"renders": renders[i], "rdram_sha256": sha(insts[i].begin_read_rdram()),
                   "hidden_sha256": sha(insts[i].begin_read_hidden_rdram())}
    return {"requests_sampled": len(picks), "of_requests": len(requests), "instances": inst}


def _check_serving_parity(sample, threads=None):
    """Second half (CPU-baseline leg): each sampled instance's frame rendered as many times through
    the CPU oracle; digests must match.  Returns the report put in the bench line."""
    import hashlib
    from concurrent.futures import ThreadPoolExecutor
    from oracle import Oracle
    from rdp_gb300 import cmdgen
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()  # noqa: E731

    def one(item):
        i, want = item
        words, rdram, _ = cmdgen.generate_stream(cmdgen.batched_instance_params(i))
        o = Oracle(8 << 20)
        o.write_rdram(rdram)
        for _ in range(want["renders"]):
            o.enqueue(words)
        ok = sha(o.rdram()) == want["rdram_sha256"] and sha(o.hidden()) == want["hidden_sha256"]
        o.close()
        return i, ok

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        results = list(ex.map(one, sorted(sample["instances"].items())))
    bad = [i for i, ok in results if not ok]
    return {"requests_sampled": sample["requests_sampled"], "of_requests": sample["of_requests"],
            "instances_checked": len(results), "renders_checked": sum(v["renders"] for v in sample["instances"].values()),
            "mismatches": bad, "passed": not bad and bool(results), "oracle_s": time.perf_counter() - t0,
            "reference": "CPU oracle, each sampled instance's frame rendered as often as it was served"}


def run_reference_batched(args):
    """The reference algorithm on the host CPU (the oracle on every host thread), same
    workload, metric and unit; each step renders every instance's frame."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    streams = _batched_streams(args.instances)
    # Each step renders half of the instances (even, then odd indices), so that a run of
    # --steps K --warmup W stays within a few minutes of CPU time.
    halves = [streams[0::2], streams[1::2]] if len(streams) > 1 else [streams]
    for k in range(args.warmup):
        _oracle_instances(halves[k % len(halves)])
    passes = frags = 0
    el = 0.0
    threads = 1
    for k in range(args.steps):
        n, p, f, t, threads = _oracle_instances(halves[k % len(halves)])
        passes += p
        frags += f
        el += t
    value = passes / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (seeded RDP command words)",
        "config": {"workload": BATCH_WORKLOAD, "instances": args.instances,
                   "primitives_per_step": sum(st[2] for st in streams)},
        "mpix_per_s": frags / el / 1e6,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "half of the instances' frames per step (even / odd indices alternating) through "
                                   "the CPU oracle (scalar restatement of the reference algorithm; the reference's "
                                   "Vulkan build needs a graphics stack), instances spread over %d host threads"
                                   % threads},
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
    ap.add_argument("--workload", default="batched", choices=["batched", "plain", "textured", "mixed"])
    ap.add_argument("--instances", type=int, default=BATCH_INSTANCES)
    ap.add_argument("--train-steps", type=int, default=8, help="sync points of online cost-model training")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serve-instances", type=int, default=256)
    ap.add_argument("--serve-window", type=float, default=0.1, help="seconds of arrivals at the configured rate")
    ap.add_argument("--serve-budget-gb", type=float, default=16.0)
    ap.add_argument("--shade-order", type=int, default=None, choices=[0, 1, 2],
                    help="shading order: 0 tile order strided, 1 per-SM queues, 2 primitive-major (default: library's)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "ours" and args.shade_order is not None:
        from rdp_gb300 import set_shade_order
        set_shade_order(args.shade_order, int(os.environ.get("LOCAL_RANK", "0")))
    if args.impl == "reference":
        (run_reference_batched if args.workload == "batched" else run_reference_single)(args)
    else:
        (run_ours_batched if args.workload == "batched" else run_ours_single)(args)


if __name__ == "__main__":
    main()
