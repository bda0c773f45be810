#!/usr/bin/env python3
"""VarDCT front-end throughput on GB300 (MP/s).

Workload: one 3840x2160 RGB8 frame from the seeded synthetic generator
(noise 4, 200 rectangles, 30 % 1/f^2 texture) at quality 75 (distance 2.35)
with the Speed::Fastest gates; one step = that frame through the whole front
end (XYB, AQ field, CfL maps, the transform search over 16x16 / 32x32 merges
and 16x8 / 8x16 re-tiling, the quant-field aggregation and matrix-header
accounting, the layout's DC/AC quantisation, tokens and per-context
histograms).  `value` is timed with CUDA events on the launching stream with
the input resident in HBM; `e2e` runs the public C ABI with host buffers
(pinned), the upload and the result download inside the timed region.
`ultrafast` times the same frame at qualities 75, 90 and 95 with the
UltraFast gates (all-DCT8, one frame each); `batch` compares, on 256 images
of log-uniform sizes (half RGBA8) at q90 with the UltraFast gates, one pass
per image against one batched pass replayed as a CUDA graph.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WIDTH, HEIGHT = 3840, 2160
QUALITIES = (75,)              # the headline workload, Speed::Fastest
SPEED = "fastest"
UF_QUALITIES = (75, 90, 95)    # the UltraFast comparison
METRIC = "VarDCT MP/s"
L2_FLUSH_BYTES = 256 << 20
INPUT_COPIES = 8               # 8 x 24.9 MB of RGB8 input, more than the 129 MB L2
BATCH_IMAGES = 256


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batch", action="store_true",
                   help="skip the 256-image plain-vs-batched comparison")
    p.add_argument("--batch-images", type=int, default=BATCH_IMAGES)
    p.add_argument("--contexts", type=int, default=3,
                   help="contexts (one stream each) the device-resident run alternates frames over")
    p.add_argument("--e2e-contexts", type=int, default=3,
                   help="contexts the end-to-end run alternates frames over")
    p.add_argument("--e2e-wide-tokens", action="store_true",
                   help="download (context, value) token pairs instead of packed AcToken words")
    p.add_argument("--c5", action="store_true",
                   help="also time one 8192x8192 RGB16 linear frame at q85 per step")
    p.add_argument("--no-refine", action="store_true",
                   help="skip the quant-field refinement timing")
    p.add_argument("--refine-steps", type=int, default=8)
    p.add_argument("--refine-weights", default="1,0.1",
                   help="the refinement's distortion mix: weight of 1 - SSIM, weight of the luma proxy")
    p.add_argument("--refine-only", action="store_true",
                   help="only run the refinement record on one context and print it (a profiler target)")
    p.add_argument("--frames-ultrafast", action="store_true",
                   help="with --frames: the UltraFast gates at q75, q90 and q95 instead of the headline")
    p.add_argument("--frames", type=int, default=0,
                   help="only run this many frames of the headline workload on one context, "
                        "untimed, and exit (the target of a profiler capture)")
    return p.parse_args()


def workload_config() -> dict:
    return {
        "workload": "VarDCT front end, 3840x2160 RGB8 sRGB, q75 (d 2.35) per step, "
                    "Speed::Fastest gates (square-merge transform search, coefficient "
                    "re-tiling, matrix-header accounting, layout coding; one pass)",
        "width": WIDTH, "height": HEIGHT, "frames_per_step": len(QUALITIES),
        "qualities": list(QUALITIES), "effort": SPEED,
        "input": "synthetic seeded generator (seed 2): cosine gradients, noise sigma 4, "
                 "200 rectangles, 30% 1/f^2 texture, 8-px checker",
        "l2": "inputs larger than L2: the timed frames read 8 device copies of the input in "
              "turn (199 MB against 129 MB of L2); no flush",
        "streams": "contexts on separate streams take the frames in turn and the steps run "
                   "back to back (--contexts, default 3 frames in flight); per-kernel times "
                   "come from a serialised pass of the same steps",
        "parallelism": "replicas only (one independent frame stream per GPU)",
    }


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the slowest replica's time); the
    value itself in a single-process run.  `device` is where the process
    group's backend keeps its tensors (a CUDA device for NCCL, None for gloo)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": reasons,
            "samples": len(self.rows),
        }


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def algorithmic_bytes(kernel: str, w: int, h: int, tokens_per_frame: float) -> float | None:
    """Bytes one launch of `kernel` must move at minimum (one frame)."""
    px = w * h
    blocks = ((w + 7) // 8) * ((h + 7) // 8)
    hist = 14850 * 128 * 4
    table = {
        # RGB8 in, three f32 planes out
        "k_xyb": px * (3 + 12),
        # three f32 planes in, one u8 per block out
        "k_adaptive_quant": px * 12 + blocks,
        # three f32 planes in; per block 192 i16 levels, 3 x i16 DC, 3 u8 and one
        # packed u32 non-zero counts, 16 B of token counts out
        "k_tile_quantize": px * 12 + blocks * (384 + 6 + 3 + 4 + 16),
        # per block the levels, packed counts, qf and token offsets in; 8-byte
        # tokens and one histogram table out
        "k_tokenize": blocks * (384 + 4 + 1 + 16) + tokens_per_frame * 8 + hist,
        # Speed::Fastest: each candidate shape reads the three planes once
        # over the positions it is priced at and writes a cost per position
        "k_cost_dct8": px * 12 + blocks * 4,
        "k_cost_16x16": px * 12 + blocks // 4 * 12,
        "k_cost_8x16": px * 12 + blocks // 2 * 4,
        "k_cost_16x8": px * 12 + blocks // 2 * 4,
        "k_cost_32x32": px * 12 + blocks // 16 * 8,
        # luma in (each site reads its own window), one bias per site out
        "k_site": px * 4 + blocks // 4 * 4 + blocks // 16 * 4,
        # costs, field and map in; map out
        "k_retile": blocks * (4 * 5 + 2),
        # the coding of the layout: each shape's launch reads the planes under
        # its transforms and writes their blocks' levels and side data; one
        # launch of each is counted as the whole frame's
        "k_layout_dct8": px * 12 + blocks * (384 + 6 + 3 + 4 + 16),
        "k_layout_16x16": px * 12 + blocks * (384 + 6 + 3 + 4 + 16),
        "k_layout_32x32": px * 12 + blocks * (384 + 6 + 3 + 4 + 16),
        "k_tokenize_layout": blocks * (384 + 4 + 1 + 16) + tokens_per_frame * 8 + hist,
    }
    return table.get(kernel)


COUNTERS = os.path.join(ROOT, "profiles", "counters_4k_q75_fastest.txt")


def counters_from_profiles(kernel: str) -> tuple[float | None, float | None]:
    """(DRAM bytes, warp instructions) of one launch of `kernel` on one
    3840x2160 q75 Speed::Fastest frame, from the committed ncu summary (its
    header gives the capture's command)."""
    if not os.path.exists(COUNTERS):
        return None, None
    for line in open(COUNTERS):
        if line.startswith(kernel + ":"):
            dram, inst = line.split(":", 1)[1].split()[:2]
            return float(dram), float(inst)
    return None, None


FP32_OPS = os.path.join(ROOT, "profiles", "fp32_ops_4k_q75_fastest.txt")


def fp32_ops_from_profiles() -> dict[str, float] | None:
    """FP32 operations per launch of each kernel of one 3840x2160 q75
    Speed::Fastest frame, from the committed ncu summary (thread-level
    FADD / FMUL / FFMA counts and their packed forms; its header gives the
    capture's command)."""
    if not os.path.exists(FP32_OPS):
        return None
    ops = {}
    for line in open(FP32_OPS):
        if line.startswith("#") or ":" not in line:
            continue
        name, rest = line.split(":", 1)
        ops[name.strip()] = float(rest.split()[0])
    return ops or None


def _synthetic():
    """The seeded image generator, loaded from its file so that the reference
    arm does not import the package (whose API loads the CUDA library)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "_bench_synthetic", os.path.join(ROOT, "jixel_gb300", "synthetic.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def cpu_baseline_run(img, threads: int | None = None, min_seconds: float = 10.0) -> dict:
    """The oracle (C restatement of the reference's scalar path) on the host cores."""
    from oracle import oracle as O

    distance_from_quality = O.distance_from_quality

    O.lib()
    cores = threads or os.cpu_count() or 1
    steps = 0
    t0 = time.perf_counter()
    while True:
        for q in QUALITIES:
            O.frontend(img, distance_from_quality(q), num_threads=cores, keep_coeffs=False,
                       speed=SPEED)
        steps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    mp = steps * len(QUALITIES) * img.shape[0] * img.shape[1] / 1e6
    return {"value": mp / dt, "unit": "MP/s", "cores": cores, "kind": "port",
            "sample": f"{steps} step(s) of {img.shape[1]}x{img.shape[0]} at "
                      f"{'/'.join('q%d' % q for q in QUALITIES)}, Speed::{SPEED.capitalize()} "
                      f"({dt:.2f} s, OpenMP over DC groups, tiles and AC groups); the C "
                      "restatement of jixel's scalar path"}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    img = _synthetic().config2_image()
    for _ in range(args.warmup):
        cpu_baseline_run(img, min_seconds=0.0)
    times = []
    for _ in range(args.steps):
        r = cpu_baseline_run(img, min_seconds=0.0)
        times.append(len(QUALITIES) * WIDTH * HEIGHT / 1e6 / r["value"])
    total = sum(times)
    value = args.steps * len(QUALITIES) * WIDTH * HEIGHT / 1e6 / total
    line = {
        "metric": METRIC, "value": value, "unit": "MP/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "MP/s", "cores": os.cpu_count() or 1,
                         "kind": "port",
                         "sample": "every step the full workload step (one 3840x2160 frame at "
                                   "q75, Speed::Fastest); the C restatement of jixel's scalar path"},
        "e2e": {"value": value, "unit": "MP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    import jixel_gb300 as J
    from jixel_gb300 import _lib as L
    from jixel_gb300 import synthetic

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    img = synthetic.config2_image()
    d_img = torch.from_numpy(img).to(dev).contiguous()
    # frames in flight: contexts on dedicated streams take the frames in
    # turn, so one frame's kernel tails overlap the next frame's
    nctx = max(2, args.contexts)
    streams = [torch.cuda.Stream(dev) for _ in range(nctx)]
    torch.cuda.set_stream(streams[0])
    ctxs = [J.FrontendContext(local) for _ in range(nctx)]
    for c, st in zip(ctxs, streams):
        assert st.cuda_stream != 0
        c.set_stream(st.cuda_stream)
    ctx = ctxs[0]
    speed = J.Speed.FASTEST if SPEED == "fastest" else J.Speed.ULTRA_FAST
    cfgs = [J.EncodeConfig(speed=speed).with_quality(q) for q in QUALITIES]
    # the autotuner picks the search kernels' launch geometry on the headline
    # frame (results do not depend on it); every context takes its choice
    autotune = None
    if speed == J.Speed.FASTEST:
        geo, tune_ms = ctx.autotune(d_img.data_ptr(), WIDTH, HEIGHT, 3, 8, cfgs[0], rounds=2)
        for c in ctxs[1:]:
            c.set_launch_geometry(geo)
        autotune = {"warps_per_cta": geo,
                    "launch_ms": {k: {str(w): round(v, 4) for w, v in t.items()}
                                  for k, t in tune_ms.items()}}
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    inputs = [d_img] + [d_img.clone() for _ in range(INPUT_COPIES - 1)]
    turn = [0]

    def step():
        for cfg in cfgs:
            ctxs[turn[0] % nctx].run_device(d_img.data_ptr(), WIDTH, HEIGHT, 3, 8, cfg)
            turn[0] += 1

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize(dev)
    tokens = []
    for cfg in cfgs:
        ctx.run_device(d_img.data_ptr(), WIDTH, HEIGHT, 3, 8, cfg)
        tokens.append(ctx.params()["num_tokens"])
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    # the K steps back to back, frames in flight on the contexts' streams;
    # the frames read their input from INPUT_COPIES device copies in turn,
    # more bytes than L2 holds, so no frame finds its input in L2
    start, end = ev(), ev()
    start.record(streams[0])
    for st in streams[1:]:
        st.wait_event(start)
    for k in range(args.steps):
        for cfg in cfgs:
            slot = turn[0] % nctx
            src = inputs[turn[0] % INPUT_COPIES]
            turn[0] += 1
            ctxs[slot].run_device(src.data_ptr(), WIDTH, HEIGHT, 3, 8, cfg)
    for st in streams[1:]:
        e_k = ev()
        e_k.record(st)
        streams[0].wait_event(e_k)
    end.record(streams[0])
    end.synchronize()
    elapsed_ms = start.elapsed_time(end)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    max_ms = max_over_ranks(elapsed_ms, dev)
    mp_per_step = len(QUALITIES) * WIDTH * HEIGHT / 1e6
    value = world * args.steps * mp_per_step / (max_ms / 1000.0)

    # per-kernel times: the same steps once more on one context, each launch
    # bracketed by CUDA events on its stream (serialised, so a launch's time
    # is its own)
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_times()
    for k in range(args.steps):
        flush.zero_()
        for cfg in cfgs:
            ctx.run_device(d_img.data_ptr(), WIDTH, HEIGHT, 3, 8, cfg)
    torch.cuda.synchronize(dev)
    ktimes = ctx.kernel_times()
    ctx.enable_kernel_timing(False)

    # roofline of the dominant kernel (event-timed launches inside the timed region)
    peaks = measured_peaks()
    dom = max(ktimes.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_n) = dom
    avg_ms = dom_ms / max(dom_n, 1)
    algo = algorithmic_bytes(dom_name, WIDTH, HEIGHT, float(np.mean(tokens)))
    hbm = algo / (avg_ms / 1000.0) / 1e9 if algo else None
    traffic, inst = counters_from_profiles(dom_name)
    hbm_line = {
        "achieved": hbm, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": (hbm / peaks["hbm_gbs"]) if hbm else None, "peak_source": peaks["source"],
        "algorithmic_bytes_per_launch": algo, "traffic": traffic,
    }
    # The search and coding kernels are issue-bound (ncu: DRAM and FP32 pipes
    # far from busy): the dominant kernel's warp instructions per launch (ncu)
    # over its event-timed launch, against the SMs' issue rate (four
    # schedulers each issuing one warp instruction a cycle at the sampled SM
    # clock).  The HBM figures stand beside it.
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if inst and sm_mhz:
        issue_peak = torch.cuda.get_device_properties(dev).multi_processor_count * 4 * sm_mhz * 1e6
        issue_rate = inst / (avg_ms / 1000.0)
        roofline = {
            "kernel": dom_name, "bound": "issue", "achieved": issue_rate, "peak": issue_peak,
            "unit": "warp instructions/s", "frac": issue_rate / issue_peak, "traffic": traffic,
            "warp_instructions_per_launch": inst, "avg_launch_ms": avg_ms,
            "share_of_kernel_time": dom_ms / sum(v[0] for v in ktimes.values()),
            "hbm": hbm_line,
        }
    else:
        roofline = dict(hbm_line, kernel=dom_name, bound="hbm", avg_launch_ms=avg_ms,
                        share_of_kernel_time=dom_ms / sum(v[0] for v in ktimes.values()))
    # the timed region ran the same launch sequence as the per-kernel pass
    launches = int(sum(v[1] for v in ktimes.values()))
    # the whole front end per frame: input bytes + 4 B per token + block side
    # data (qf, strategy, 3 DC levels: 0.125 B/px) + CfL maps (2 B per 4096
    # px) + one histogram set (14850 x 128 x 4 B), over the frame's summed
    # kernel time
    px = WIDTH * HEIGHT
    fe_bytes = (3 * px + 4 * float(np.mean(tokens)) + 0.125 * px + 2 * px / 4096
                + L.NUM_FINE_AC_CONTEXTS * L.ALPHABET_SIZE * 4)
    fe_ms = sum(v[0] for v in ktimes.values()) / (args.steps * len(QUALITIES))
    roofline["frontend"] = {
        "algorithmic_bytes_per_frame": fe_bytes, "kernel_ms_per_frame": fe_ms,
        "achieved": fe_bytes / (fe_ms / 1000.0) / 1e9,
        "frac": fe_bytes / (fe_ms / 1000.0) / 1e9 / peaks["hbm_gbs"],
    }
    # FP32 work: the operations the frame's kernels executed (ncu counts of
    # the same frame) over the frame's summed kernel time, against the CUDA
    # cores' nominal FP32 rate (128 lanes an SM, an FMA two operations, at the
    # sampled SM clock); no measured FP32 peak exists for this machine
    ops = fp32_ops_from_profiles()
    if ops and sm_mhz:
        total_ops = sum(ops.values())
        fp32_peak = torch.cuda.get_device_properties(dev).multi_processor_count * 128 * 2 * sm_mhz * 1e6 / 1e12
        achieved = total_ops / (fe_ms / 1000.0) / 1e12
        top = max(ops.items(), key=lambda kv: kv[1] / max(ktimes.get(kv[0], (1e30, 1))[0], 1e-9))
        roofline["fp32"] = {
            "ops_per_frame": total_ops, "kernel_ms_per_frame": fe_ms, "achieved": achieved,
            "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
            "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2 at the sampled SM clock)",
            "densest_kernel": top[0],
        }

    ultrafast = run_ultrafast(ctxs, streams, flush, d_img, args, dev)
    c5 = run_c5(ctxs, streams, flush, args, dev) if args.c5 else None
    batch = None
    if not args.no_batch:
        batch = run_batch(ctx, streams[0], flush, args, world, dev)

    refine = None
    if not args.no_refine:
        refine = run_refine(ctx, streams[0], args, dev)

    # end to end through the public C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(ctx, img, cfgs, args, world, dev, autotune["warps_per_cta"] if autotune else None)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_run(img)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "MP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(), "impl": "gb300",
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clocks,
            "kernels_ms_per_step": {k: v[0] / args.steps for k, v in sorted(ktimes.items())},
            "tokens_per_frame": [int(x) for x in tokens],
            "batch": batch,
            "autotune": autotune,
            "ultrafast": ultrafast,
            "c5": c5,
            "refine": refine,
        }
        print(json.dumps(line), flush=True)
    for c in ctxs:
        c.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_ultrafast(ctxs, streams, flush, d_img, args, dev) -> dict:
    """The same frame at q75, q90 and q95 with the UltraFast gates (all-DCT8
    layout), three frames per step over the contexts in turn, CUDA events on
    the streams, L2 flushed between steps."""
    import torch

    import jixel_gb300 as J

    cfgs = [J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(q) for q in UF_QUALITIES]
    nctx = len(ctxs)
    turn = [0]

    def step():
        for cfg in cfgs:
            ctxs[turn[0] % nctx].run_device(d_img.data_ptr(), WIDTH, HEIGHT, 3, 8, cfg)
            turn[0] += 1

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize(dev)
    total = 0.0
    for _ in range(args.steps):
        flush.zero_()
        s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(streams[0])
        for st in streams[1:]:
            st.wait_event(s0)
        step()
        for st in streams[1:]:
            ek = torch.cuda.Event(enable_timing=True)
            ek.record(st)
            streams[0].wait_event(ek)
        e0.record(streams[0])
        e0.synchronize()
        total += s0.elapsed_time(e0)
    mp = len(cfgs) * WIDTH * HEIGHT / 1e6
    return {"workload": "3840x2160 RGB8 at q75/q90/q95, UltraFast gates (all-DCT8 layout), "
                        "three frames per step", "value": args.steps * mp / (total / 1000.0),
            "unit": "MP/s", "ms_per_step": total / args.steps}


def run_refine(ctx, stream, args, dev) -> dict:
    """Quant-field refinement of one 1920x1080 RGB8 frame (the 3840x2160
    generator, seed 4: 240 x 135 blocks) after its UltraFast pass at q90:
    `--refine-steps` Adam steps (loss, gradient by the adjoint kernels,
    update) after one untimed step, CUDA events on the context's stream
    around the steps, each of which reads its loss back to the host.  Then
    the refined field is rounded and coded: the model's distortion at that
    field and the pass's AC bits (`ac_bits_estimate`) against the adaptive
    field's."""
    import torch

    import jixel_gb300 as J
    from jixel_gb300 import synthetic

    img = synthetic.config4_image()
    h, w = img.shape[:2]
    cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90)
    lr = 0.05
    base = ctx.frontend(img, cfg, coefficients=False)
    xb, yb = ctx.refine_begin()
    weights = tuple(float(v) for v in args.refine_weights.split(","))
    ctx.refine_weights(*weights)
    # lambda at the pass's own rate-distortion slope: the steps trade bits
    # between blocks at the exchange rate the frame already has
    lam = ctx.refine_rate_slope(w * h)
    first = ctx.refine_step(lam, lr)
    ctx.refine_theta(np.zeros((yb, xb), np.float32))  # restart from theta = 0
    torch.cuda.synchronize(dev)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    s.record(stream)
    hist = [ctx.refine_step(lam, lr) for _ in range(args.refine_steps)]
    e.record(stream)
    e.synchronize()
    wall = time.perf_counter() - t0
    final, _ = ctx.refine_eval(lam)
    ms = s.elapsed_time(e) / args.refine_steps
    # per-kernel times of one more step; algorithmic bytes per launch: the
    # fused SSIM kernel reads the source and decoded planes and writes the
    # gradient (12 B per pixel and channel at its scale); the forward reads the
    # source coefficients and writes the decoded XYB and linear planes (2304 B
    # per block), the backward reads coefficients, decoded XYB and the two
    # finest gradients (2496 B per block)
    theta = ctx.refine_theta()
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_times()
    ctx.refine_step(lam, lr)
    kt = {k: v for k, v in ctx.kernel_times().items() if k.startswith("k_refine")}
    ctx.enable_kernel_timing(False)
    nb = xb * yb
    px = [w * h, (w // 2) * (h // 2), (w // 4) * (h // 4)]
    algo = {"k_refine_forward": 2304.0 * nb, "k_refine_backward": 2496.0 * nb,
            "k_refine_ssim": 36.0 * sum(px)}
    kernels = {}
    for k, v in sorted(kt.items()):
        kernels[k] = {"ms": v[0], "launches": v[1]}
        if k in algo:
            kernels[k]["algorithmic_gbs"] = algo[k] / (v[0] / 1000.0) / 1e9
    ctx.refine_theta(theta)
    coded = _refined_field_report(ctx, img, cfg, base, ctx.refine_field(), lam)
    # the same refinement with the reference's own luma proxy as the
    # distortion (weights 0, 1), from theta = 0 at that measure's slope
    ctx.refine_weights(0.0, 1.0)
    ctx.refine_theta(np.zeros((yb, xb), np.float32))
    lam_p = ctx.refine_rate_slope(w * h)
    for _ in range(args.refine_steps):
        ctx.refine_step(lam_p, lr)
    coded_proxy = _refined_field_report(ctx, img, cfg, base, ctx.refine_field(), lam_p)
    coded_proxy["lambda"] = lam_p
    ctx.refine_weights(*weights)
    return {"workload": f"{w}x{h} RGB8 (seed 4) q90 UltraFast pass, {nb} blocks, Adam lr {lr}, "
                        f"lambda {lam:.4g} (the pass's rate-distortion slope), distortion "
                        f"{weights[0]} x (1 - SSIM at 3 scales) + {weights[1]} x luma proxy, rate model",
            "weights": weights,
            "steps": args.refine_steps, "ms_per_step": ms, "wall_ms_per_step": 1000.0 * wall / args.refine_steps,
            "megapixels_per_s": w * h / 1e6 / (ms / 1000.0),
            "loss_first": hist[0][0], "loss_final": final[0], "distortion_first": hist[0][1],
            "distortion_final": final[1], "model_bits_first": hist[0][2], "model_bits_final": final[2],
            "untimed_first_step_loss": first[0],
            "coded": coded, "coded_luma_proxy_objective": coded_proxy,
            "kernels": kernels}


def _refined_field_report(ctx, img, cfg, base, field, lam) -> dict:
    """A refined field as coded, under the context's distortion weights: the
    model's distortion at theta = log(field / qf) and the pass's AC bits
    (`ac_bits_estimate`: per-context symbol entropy + the tokens' raw bits)
    against the adaptive field's, and against uniform rescalings of the
    adaptive field at the same distortion (the two integer fields that
    bracket it, coded, their rates interpolated); then both distortion
    measures (1 - SSIM, the luma proxy) at every field."""
    import jixel_gb300 as J

    h, w = img.shape[:2]
    qf = base.quant_field.astype(np.float64)

    def at_field(f):
        ctx.refine_theta(np.log(f.astype(np.float64) / qf).astype(np.float32))
        return ctx.refine_eval(lam)[0]

    def uniform(c):  # a larger field quantises finer
        return np.clip(np.rint(qf * np.exp(c)), 1, 255).astype(np.uint8)

    d0, d1 = at_field(base.quant_field)[1], at_field(field)[1]
    lo, hi = -1.0, 1.0
    for _ in range(20):
        mid = 0.5 * (lo + hi)
        if at_field(uniform(mid))[1] < d1:
            hi = mid
        else:
            lo = mid
    brackets = []
    for c in (lo, hi):
        f = uniform(c)
        brackets.append((c, at_field(f)[1], J.ac_bits_estimate(ctx.frontend_with_field(img, cfg, f, coefficients=False))))
    (_, d_lo, b_lo), (_, d_hi, b_hi) = brackets
    t = 0.0 if d_lo == d_hi else (d1 - d_hi) / (d_lo - d_hi)
    bits_uniform = b_hi + t * (b_lo - b_hi)
    bits0 = J.ac_bits_estimate(base)
    bits1 = J.ac_bits_estimate(ctx.frontend_with_field(img, cfg, field, coefficients=False))
    measures = {}
    ws, wp = ctx.refine_weights_now
    for name, wts in (("ssim", (1.0, 0.0)), ("luma_proxy", (0.0, 1.0))):
        ctx.refine_weights(*wts)
        measures[name] = {"adaptive_field": at_field(base.quant_field)[1], "refined_field": at_field(field)[1],
                          "uniform_brackets": [at_field(uniform(c))[1] for c, _, _ in brackets]}
    ctx.refine_weights(ws, wp)
    return {"distortion_adaptive_field": d0, "distortion_refined_field": d1,
            "ac_bpp_adaptive_field": bits0 / (w * h), "ac_bpp_refined_field": bits1 / (w * h),
            "uniform_scale_same_distortion": {
                "brackets": [{"log_scale": c, "distortion": d, "ac_bpp": b / (w * h)} for c, d, b in brackets],
                "ac_bpp_interpolated": bits_uniform / (w * h)},
            "refined_over_uniform_bits": bits1 / bits_uniform,
            "measures": measures}


def run_c5(ctxs, streams, flush, args, dev) -> dict:
    """One 8192x8192 RGB 16-bit linear frame (50 % 1/f^2 texture) at q85 per
    step, pixels resident in HBM, the two contexts taking steps in turn."""
    import torch

    import jixel_gb300 as J
    from jixel_gb300 import synthetic

    size = 8192
    img = synthetic.config5_image(size)
    d_img = torch.from_numpy(img.reshape(-1).view(np.uint8)).to(dev)
    cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST, transfer=J.TransferFunction.LINEAR).with_quality(85)

    def frame(k):
        ctxs[k % 2].run_device(d_img.data_ptr(), size, size, 3, 16, cfg)

    for k in range(max(args.warmup, 1)):
        frame(k)
    torch.cuda.synchronize(dev)
    total = 0.0
    for k in range(args.steps):
        flush.zero_()
        s, eb, e = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        s.record(streams[0])
        streams[1].wait_event(s)
        frame(k)
        eb.record(streams[1])
        streams[0].wait_event(eb)
        e.record(streams[0])
        e.synchronize()
        total += s.elapsed_time(e)
    mp = size * size / 1e6
    # the frame's quant-field refinement: 4 Adam steps over its 1,048,576
    # blocks, the EPF at the frame's own loop-filter setting
    ctx = ctxs[0]
    ctx.run_device(d_img.data_ptr(), size, size, 3, 16, cfg)
    epf_iters = ctx.params()["epf_iters"]
    xb, yb = ctx.refine_begin()
    lam = ctx.refine_rate_slope(size * size)
    ctx.refine_step(lam, 0.05)  # untimed
    ctx.refine_theta(np.zeros((yb, xb), np.float32))
    torch.cuda.synchronize(dev)
    rs, re = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rs.record(streams[0])
    hist = [ctx.refine_step(lam, 0.05) for _ in range(4)]
    re.record(streams[0])
    re.synchronize()
    final, _ = ctx.refine_eval(lam)
    # the same 4 steps through the monotone driver (a step that raises the
    # rounded loss is taken back and the learning rate halved)
    _, _, mono = ctx.refine(steps=4, rate_lambda=lam, learning_rate=0.05, monotone=True)
    return {"workload": "8192x8192 RGB 16-bit linear, q85 (d 1.45), UltraFast gates, one frame "
                        "per step", "value": args.steps * mp / (total / 1000.0), "unit": "MP/s",
            "ms_per_frame": total / args.steps,
            "refine": {"steps": 4, "blocks": xb * yb, "ms_per_step": rs.elapsed_time(re) / 4,
                       "epf_stages": epf_iters, "loss_first": hist[0][0],
                       "loss_final": final[0], "loss_final_monotone": mono[0]}}


def run_batch(ctx, stream, flush, args, world, dev) -> dict:
    """256 images of log-uniform sizes 64x64..2048x1536 (odd ones RGBA8), q90:
    one pass per image (`plain`) against one pass for the whole set
    (`batched`: one launch per stage over every frame, replayed as a CUDA
    graph).  Pixels are resident in HBM for both; CUDA events time each step
    on the launching stream."""
    import torch

    import jixel_gb300 as J
    from jixel_gb300 import synthetic

    imgs = synthetic.config3_batch(args.batch_images)
    mp = sum(i.shape[0] * i.shape[1] for i in imgs) / 1e6
    cfg = J.EncodeConfig(speed=J.Speed.ULTRA_FAST).with_quality(90)
    d_imgs = [torch.from_numpy(i.reshape(-1)).to(dev) for i in imgs]
    torch.cuda.synchronize(dev)

    def plain_step():
        for img, d in zip(imgs, d_imgs):
            h, w, ch = img.shape
            ctx.run_device(d.data_ptr(), w, h, ch, 8, cfg)

    b = ctx.batch(pixels_on_device=True)
    for img, d in zip(imgs, d_imgs):
        h, w, ch = img.shape
        b.add_device(d.data_ptr(), w, h, ch, 8, cfg, keep=d)

    def batched_step():
        b.run(use_graph=True)

    def timed(fn) -> float:
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        total = 0.0
        for _ in range(args.steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            torch.cuda.synchronize(dev)
            total += s.elapsed_time(e)
        return max_over_ranks(total, dev)

    plain_ms = timed(plain_step)
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_times()
    b.run(use_graph=False)  # per-kernel times of one batched pass (graphs carry no events)
    ktimes = ctx.kernel_times()
    ctx.enable_kernel_timing(False)
    batched_ms = timed(batched_step)
    b.close()
    plain = world * args.steps * mp / (plain_ms / 1000.0)
    batched = world * args.steps * mp / (batched_ms / 1000.0)
    return {
        "workload": f"{len(imgs)} images, log-uniform 64x64..2048x1536, half RGB8 half RGBA8, "
                    "q90, UltraFast gates",
        "megapixels_per_step": mp, "unit": "MP/s",
        "plain": {"value": plain, "ms_per_step": plain_ms / args.steps,
                  "launches_per_step": 7 * len(imgs)},
        "batched": {"value": batched, "ms_per_step": batched_ms / args.steps,
                    "launches_per_step": 7, "cuda_graph": True},
        "batched_over_plain": batched / plain,
        "batched_kernels_ms": {k: v[0] for k, v in sorted(ktimes.items())},
    }


def run_e2e(ctx, img, cfgs, args, world, dev, geometry=None):
    """End to end through the public C ABI: every frame is uploaded from
    pinned host memory and its outputs (maps, DC levels, tokens, group
    offsets, histograms) land in pinned host memory, all inside the timed
    region.  Tokens come in the groups' storage form (AcTokens: one word per
    token), or as (context, value) pairs with --e2e-wide-tokens.  The caller
    pipelines frames over several contexts with jxg_frontend_enqueue /
    jxg_frontend_wait, so one frame's transfers overlap another's kernels."""
    import ctypes

    import torch

    import jixel_gb300 as J
    from jixel_gb300 import _lib as L
    from jixel_gb300 import frame_info

    lib = L.load()
    fi = frame_info(WIDTH, HEIGHT)
    h_img = torch.empty(img.size, dtype=torch.uint8, pin_memory=True)
    h_img.numpy()[:] = img.reshape(-1)
    nctx = max(1, args.e2e_contexts)
    ctxs = [J.FrontendContext(dev.index or 0) for _ in range(nctx)]
    if geometry:
        for c in ctxs:
            c.set_launch_geometry(geometry)
    packed = not args.e2e_wide_tokens
    outs = [J.PinnedOutputs(WIDTH, HEIGHT, packed=packed) for _ in range(nctx)]
    c_cfgs = [c._c() for c in cfgs]
    nb = fi.xsize_blocks * fi.ysize_blocks
    nt = fi.xsize_tiles * fi.ysize_tiles
    # quant field, strategy map, CfL maps, DC levels, group offsets, histograms
    fixed_d2h = (nb + nb + 2 * nt + 6 * nb + (fi.num_groups + 1) * 8
                 + L.NUM_FINE_AC_CONTEXTS * L.ALPHABET_SIZE * 4)
    state = {"pending": [False] * nctx, "d2h": 0, "k": 0}

    def finish(slot):
        if state["pending"][slot]:
            st = lib.jxg_frontend_wait(ctxs[slot].handle)
            if st:
                raise RuntimeError(f"jxg_frontend_wait status {st}")
            state["pending"][slot] = False
            o = outs[slot]
            if packed:
                state["d2h"] += fixed_d2h + int(o.packed_offsets[-1]) * 4 + (fi.num_groups + 1) * 8
            else:
                state["d2h"] += fixed_d2h + o.params.num_tokens * 8

    def step():
        for c in c_cfgs:
            slot = state["k"] % nctx
            state["k"] += 1
            finish(slot)
            st = lib.jxg_frontend_enqueue(ctxs[slot].handle, ctypes.c_void_p(h_img.data_ptr()),
                                          WIDTH, HEIGHT, 3, 8, ctypes.byref(c),
                                          ctypes.byref(outs[slot].params), ctypes.byref(outs[slot].c))
            if st:
                raise RuntimeError(f"jxg_frontend_enqueue status {st}")
            state["pending"][slot] = True

    for _ in range(max(args.warmup, 1)):
        step()
    for slot in range(nctx):
        finish(slot)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    state["d2h"] = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    for slot in range(nctx):
        finish(slot)
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    dt = max_over_ranks(dt, dev)
    for c in ctxs:
        c.close()
    value = world * args.steps * len(QUALITIES) * WIDTH * HEIGHT / 1e6 / dt
    return {"value": value, "unit": "MP/s", "h2d_bytes_per_step": len(QUALITIES) * img.size,
            "d2h_bytes_per_step": int(state["d2h"] / args.steps),
            "path": f"jxg_frontend_enqueue / jxg_frontend_wait (C ABI), {nctx} contexts taking "
                    "frames in turn: pinned host RGB in; quant field, strategy and CfL maps, DC "
                    "levels, tokens "
                    f"({'packed AcToken words' if packed else 'context/value pairs'}), group "
                    "offsets and histograms out to pinned host memory"}


def run_frames(args):
    """`--frames K`: K frames of the headline workload, one after another on
    one context (for ncu: its launches repeat every frame)."""
    import torch

    import jixel_gb300 as J
    from jixel_gb300 import synthetic

    img = synthetic.config2_image()
    d_img = torch.from_numpy(img).cuda().contiguous()
    ctx = J.FrontendContext(0)
    speed = J.Speed.FASTEST if SPEED == "fastest" else J.Speed.ULTRA_FAST
    qualities = QUALITIES
    if args.frames_ultrafast:
        speed, qualities = J.Speed.ULTRA_FAST, UF_QUALITIES
    for k in range(args.frames):
        for q in qualities:
            ctx.run_device(d_img.data_ptr(), WIDTH, HEIGHT, 3, 8, J.EncodeConfig(speed=speed).with_quality(q))
    torch.cuda.synchronize()
    ctx.close()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.frames:
        run_frames(args)
    elif args.refine_only:
        import torch

        import jixel_gb300 as J
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        ctx = J.FrontendContext(0)
        ctx.set_stream(stream.cuda_stream)
        print(json.dumps({"refine": run_refine(ctx, stream, args, torch.device("cuda", 0))}), flush=True)
        ctx.close()
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
