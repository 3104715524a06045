#!/usr/bin/env python3
"""Benchmark: 1080p stylised frames/s of PaintTween's offset-field synthesis.

Workload (one "step"): the 24-frame 1920x1080 clip with a 1024x1024 exemplar
(6 moving discs, 4 object IDs), patch radius 3, 5 pyramid levels, 6
iterations per level, histogram term on, forward + backward consecutive
passes (FMBM_RM) -- synthesised end to end by the CUDA library.

  value  frames/s with the frame pyramids already resident in HBM (device
         time from CUDA events on the library's stream, max over ranks)
  e2e    frames/s through the C ABI with host buffers: every step uploads
         the 24 frames (H2D, pyramids built on the device) and reads back
         every frame's output and offsets (D2H)
  roofline  the dominant kernel (propagate) from per-launch CUDA events and
         counted patch-distance evaluations of the same timed steps
  cpu_baseline  the CPU oracle (a scalar C restatement of the reference's
         kernels; the reference has no CPU path) on a bounded sample

  ref_kernels_gpu  the reference's own CUDA kernels and host wrappers,
         compiled unchanged over texture objects (oracle/refport), on the
         first frames of the same clip on the same GPU

`--impl reference` times the CPU restatement of the reference's kernels (the
reference has no CPU path), each step one bounded sample of a temporal
frame; its frames/s is extrapolated from that sample's evaluation rate.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from painttween_gb300 import _abi, synthetic  # noqa: E402

WORKLOAD = "clip1080p"
METRIC = "1080p stylized frames/s"
UNIT = "frames/s"

# DRAM bytes (read + write) per level pixel of one kt_propagate_q launch: the
# ncu capture of a level-0 temporal launch of this workload (1920x1080 level,
# 340.1 MB read + 64.9 MB written) summarised in
# profiles/kt_energy_kernels_clip1080p.md.  The exemplar planes stay in L2,
# so DRAM traffic follows the staged pixel-side planes, i.e. the level area.
PROPAGATE_DRAM_BYTES_PER_PIXEL = (340.1e6 + 64.9e6) / (1920 * 1080)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Replicas only: each rank synthesises its own clip on its own GPU; a
    gloo group supplies the barrier and the max over ranks."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([float(v)])
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


# ---------------------------------------------------------------------------
# inputs and the analytic evaluation count of the schedule
# ---------------------------------------------------------------------------

def make_inputs(cfg, frames, seed=2026):
    ex = synthetic.make_exemplar(cfg["ew"], cfg["eh"], seed=seed)
    clip = synthetic.make_clip(cfg["w"], cfg["h"], cfg["discs"], frames, seed=seed + 1)
    return ex, clip


def active_pixels(clip, levels, cull):
    """Non-culled pixels (image DT <= cull) per frame and level, with the DT
    pyramid built like the reference (2x2 average)."""
    out = []
    for fr in clip:
        dt = fr["dist_trans"].astype(np.float32)
        per = []
        for lv in range(levels):
            per.append(int((dt <= np.float32(cull)).sum()))
            h, w = dt.shape
            a = dt[0:h - h % 2:2, 0:w - w % 2:2] + dt[0:h - h % 2:2, 1:w - w % 2:2]
            a = a + dt[1:h - h % 2:2, 0:w - w % 2:2]
            dt = ((a + dt[1:h - h % 2:2, 1:w - w % 2:2]) * np.float32(0.25)).astype(np.float32)
        out.append(per)
    return out


def scatter_samples(ew, eh, count=25):
    """Candidates of the scatter chain: dist = 0.9^i * max(w, h) (float32)
    while 0.9 * dist >= 10, at most scatterSamplesCount."""
    f = np.float32
    dist, n = f(max(ew, eh)), 0
    while n < count and f(dist * f(0.9)) >= f(10.0):
        dist = f(dist * f(0.9))
        n += 1
    return n


def evals_per_step(p, cfg, act, frames):
    """Patch-distance evaluations of one clip synthesis (exemplar DT 0 and
    alpha 1: no candidate is rejected before evaluation)."""
    total = 0
    it = p.iterations
    for lv in range(p.levels):
        s = scatter_samples(cfg["ew"] >> lv, cfg["eh"] >> lv, p.scatterSamplesCount)
        per_px = it * 9 * (4 + 1) + (it - 1) * ((s + 1) + 1)  # propagates/scatters + their syncs
        for f in range(frames):
            a = act[f][lv]
            # pass 0: random/upsample sync + (merge sync) + final sync
            extra0 = 2 if (f == 0) else (3 if lv < p.levels - 1 else 1)
            total += a * (per_px + extra0)
            if f != frames - 1:  # pass 1 (backward): merge sync + final sync
                total += a * (per_px + 2)
    return total


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
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
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU arms
# ---------------------------------------------------------------------------

def cpu_sample(cfg, p, ex, clip, threads, passes=1):
    """The CPU oracle on `passes` level-0 propagate passes (jump 8) of frame 1
    of the clip at full size, with its temporal terms: frame 0 is randomised
    and propagated once, then frame 1 takes the forward-advected offsets and
    the random merge, as in the forward consecutive pass.  Returns
    (evaluations/s, description, seconds of the timed passes)."""
    from oracle import oracle as O
    o = O.Oracle(cfg["w"], cfg["h"], cfg["ew"], cfg["eh"], 1, threads=threads)
    q = p.copy()
    q.direction = _abi.FORWARD
    q.filterMode = _abi.FILTER_EXACT  # a CPU has no texture unit: bilinear weights in FP32
    o.set_params(q)
    sp = O.style_pyramids(ex)
    fps = [O.frame_pyramids(clip[0]), O.frame_pyramids(clip[1])]
    o.load_style_level([sp], 0)
    o.reset_advected()
    for f in (0, 1):
        fp = fps[f]
        if f:
            o.flip()
        o.load_frame_level(fp, 0)
        rnd = O.random_level(0, 0, cfg["ew"], cfg["eh"], fp["rgba"][0], fp["orient"][0], sp["output"][0],
                             sp["orient"][0])
        o.upload_random(rnd)
        if f == 0:
            o.randomize_offsets(0)
            o.propagate(0, 8)
        else:
            o.advect(0, 1, True, 0)
            o.merge_randomly(0, True, 0.5, False)
            o.sync(0, 0)
    act = int((fps[1]["dt"][0] <= np.float32(p.distTransCull)).sum())
    lib = O.lib()
    t0 = time.perf_counter()
    for _ in range(passes):
        lib.pto_propagate(o.h, 0, 8)
    dt = time.perf_counter() - t0
    o.close()
    evals = 4 * act * passes
    desc = ("%d level-0 propagate pass(es) (4 candidates x %d active pixels, r=%d, temporal terms on, bilinear "
            "in FP32) of frame 1 of the 1920x1080 clip on %d thread(s)" % (passes, act, p.residualWindowSize, threads))
    return evals / dt, desc, dt


def run_reference(args, dist):
    """The reference arm: the CPU restatement of the reference's kernels (the
    reference has no CPU path; its CUDA kernels are timed on the GPU in our
    arm's `ref_kernels_gpu`).  Each step is one bounded sample, a level-0
    propagate pass of a temporal frame on every host thread; frames/s is
    that rate over the schedule's evaluations per frame (extrapolated), and
    ms_per_step is the time the step actually took."""
    if args.gpus != dist.ws:
        raise SystemExit("--gpus %d but %d rank(s) launched" % (args.gpus, dist.ws))
    cfg = synthetic.config(WORKLOAD)
    p = cfg["params"]
    frames = args.frames or cfg["frames"]
    if dist.rank != 0:
        return 0
    threads = os.cpu_count() or 1
    ex, clip = make_inputs(cfg, max(frames, 2))
    act = active_pixels(clip, p.levels, p.distTransCull)
    per_frame = evals_per_step(p, cfg, act, frames) / frames
    rates, secs = [], []
    desc = ""
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rate, desc, _ = cpu_sample(cfg, p, ex, clip, threads)
        if i >= args.warmup:
            rates.append(rate)
            secs.append(time.perf_counter() - t0)
    rate = float(np.mean(rates))
    fps = rate / per_frame
    line = {
        "impl": "reference", "metric": METRIC, "value": fps, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(secs)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "frames": frames, "image": "1920x1080", "exemplar": "1024x1024",
                   "patch_radius": p.residualWindowSize, "levels": p.levels, "iterations": p.iterations,
                   "scheme": "FMBM_RM", "histogram": True, "parallelism": "host threads"},
        "extrapolated": True,
        "cpu_baseline": {"value": fps, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": desc + " per step (set-up included in ms_per_step); frames/s = evaluations/s "
                                          "/ evaluations per frame of the schedule"},
        "e2e": {"value": fps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "evals_per_s": rate, "evals_per_frame": per_frame,
    }
    print(json.dumps(line))
    return 0


def ref_kernels_gpu(frames=2):
    """The reference's own CUDA kernels and TexSynth host wrappers (compiled
    unchanged over texture objects, oracle/refport) on the first `frames`
    frames of the benchmark clip at its full settings, on this GPU: wall time
    of the reference's per-frame call sequence, with its host-side random
    pyramid and its synchronisation after every launch, EXR files excluded.
    None when the port's sources are not staged."""
    try:
        from oracle.refport import build as rb
        if rb.build() is None:
            return {"unavailable": "reference port not staged (oracle/_ref/refport_src absent)"}
        from oracle.refport import port as RP
    except Exception as e:
        return {"unavailable": "reference port does not build: %s" % str(e).splitlines()[0][:200]}
    cfg = synthetic.config(WORKLOAD)
    p = cfg["params"]
    ex, clip = make_inputs(cfg, frames)
    d = RP.RefPortDriver(p, [ex], clip)
    t0 = time.perf_counter()
    d.render(0, frames - 1)
    wall = time.perf_counter() - t0
    d.o.close()
    return {"value": frames / wall, "unit": UNIT, "frames": frames, "seconds": wall,
            "what": "the reference's CUDA kernels and host wrappers (texSynth_kernel.cu, convolution.cu, "
                    "compiled unchanged for sm_103a) on the first %d frames of the clip, all 5 levels, "
                    "FMBM_RM forward and backward; wall time, EXR I/O excluded" % frames}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def gather_ceilings(device):
    """L2-resident 32-byte record gather rates (GB/s) on this GPU: random
    per lane and coherent per warp (pt_measure_gather)."""
    import ctypes
    from painttween_gb300._lib import lib
    out = {}
    for name, coh in (("random", 0), ("coherent", 1)):
        v = ctypes.c_double(0.0)
        if lib().pt_measure_gather(device, coh, ctypes.byref(v)) == 0:
            out[name] = v.value
    return out


def run_ours(args, dist):
    from painttween_gb300 import Synthesizer, host_array
    from painttween_gb300 import build as B
    if args.gpus != dist.ws:
        raise SystemExit("--gpus %d but %d rank(s) launched: start N > 1 with torch.distributed.run" %
                         (args.gpus, dist.ws))
    B.build()
    cfg = synthetic.config(WORKLOAD)
    p = cfg["params"]
    p.filterMode = _abi.FILTER_EXACT if args.filter == "exact" else _abi.FILTER_TEXTURE
    frames = args.frames or cfg["frames"]
    device = dist.local
    ex, clip = make_inputs(cfg, frames, seed=2026 + dist.rank)
    s = Synthesizer(device=device)
    s.setup(p, cfg["w"], cfg["h"], cfg["ew"], cfg["eh"], 1)
    if args.generic_kernels:
        s.set_tiled_kernels(False)  # same results, one-thread-per-pixel kernels (profiling them)
    s.set_tma_staging(args.staging == "tma")
    s.set_propagate_lanes(args.propagate_lanes)
    s.set_style(0, ex["base"], ex["output"], ex["orient_tensor"], ex["dist_trans"], ex["object_ids"])
    for i, fr in enumerate(clip):
        s.set_frame_dict(i, fr)

    def render():
        s._check(__import__("painttween_gb300._lib", fromlist=["lib"]).lib().pt_synthesize_animation(
            s.h, 0, frames - 1, None, None), "pt_synthesize_animation")

    gc = gather_ceilings(device)
    for _ in range(args.warmup):
        render()
    s.synchronize()
    # Evaluation and tap counts: one untimed step with the device-side
    # counters (atomics inside the kernels).  The synthesis is deterministic,
    # so every step repeats these counts exactly.
    s.set_profiling(_abi.PROFILE_COUNTERS)
    render()
    counts = {k: s.kernel_stats(k) for k in range(4)}
    s.set_profiling(0)
    dist.barrier()

    # timed steps: an event pair around every launch gives the kernels'
    # durations; no counters run here
    clocks = Clocks(device)
    clocks.start()
    s.set_profiling(_abi.PROFILE_TIMING)
    l0 = s.kernel_launches
    times = []
    for _ in range(args.steps):
        s.timer_record(0)
        render()
        s.timer_record(1)
        times.append(s.timer_elapsed(0, 1))
    launches = s.kernel_launches - l0
    stats = {k: s.kernel_stats(k) for k in range(4)}
    for k in stats:
        for f in ("energy_evals", "taps", "temporal_taps"):
            stats[k][f] = counts[k][f] * args.steps
    s.set_profiling(0)
    ck = clocks.stop()
    total_ms = dist.max(sum(times))
    dist.barrier()

    # end to end through the C ABI with host buffers: every step uploads the
    # clip's inputs from page-locked host memory (pt_set_frame builds the
    # pyramids on the device), synthesises, and reads every frame's output
    # and offsets back into page-locked host memory (pt_get_frame_result)
    e2e_times = []
    keys = ("rgba", "orient_tensor", "dist_trans", "object_ids", "vel_fwd", "vel_bwd", "scale")
    pinned = []
    for fr in clip:
        d = {}
        for key in keys:
            d[key] = host_array(fr[key].shape, fr[key].dtype)
            d[key][...] = fr[key]
        pinned.append(d)
    h2d = sum(d[key].nbytes for d in pinned for key in keys)
    h, w = cfg["h"] >> _abi.output_level(p), cfg["w"] >> _abi.output_level(p)
    outs = [(host_array((h, w, 4), np.float32), host_array((h, w), _abi.PATCH_DTYPE)) for _ in range(frames)]
    d2h = sum(a.nbytes + o.nbytes for a, o in outs)
    e2e_steps = args.steps if args.e2e_steps < 0 else args.e2e_steps
    s.set_profiling(_abi.PROFILE_TIMING)  # the profiling state of the timed steps
    for _ in range(e2e_steps):
        s.synchronize()
        t0 = time.perf_counter()
        s.timer_record(2)
        for i, d in enumerate(pinned):
            s.set_frame_dict(i, d)
        render()
        for f, (a, o) in enumerate(outs):
            s.get_frame_result(f, a, o)
        s.timer_record(3)
        e2e_times.append(max(s.timer_elapsed(2, 3), 1000.0 * (time.perf_counter() - t0)))
    s.set_profiling(0)
    e2e_ms = dist.max(float(np.mean(e2e_times)) * args.steps) if e2e_times else None

    # roofline of the dominant kernel (propagate)
    st = stats[_abi.KERNEL_PROPAGATE]
    r = p.residualWindowSize
    K = (2 * r + 1) ** 2
    # algorithmic work per evaluation: 2 exemplar float4 samples per tap
    # (32 B, ~84 flops) + 16 B at the centre; temporal taps add 2 samples and
    # 3 SSDs (+32 B, +84 flops)
    n_launch = max(st["launches"], 1)
    evals_per_launch = st["energy_evals"] / n_launch
    # algorithmic bytes: every evaluation over all K taps (32 K + 16 B), and
    # the temporal ones 32 K more; the early exit and the change tracking
    # skip part of them, so the bytes of the work done are kept beside
    temporal_frac = st["temporal_taps"] / max(st["taps"], 1)
    alg_bytes_per_launch = (st["energy_evals"] * (32 * K + 16) +
                            st["energy_evals"] * temporal_frac * 32 * K) / n_launch
    bytes_per_launch = (32 * st["taps"] + 16 * st["energy_evals"] + 32 * st["temporal_taps"]) / n_launch
    flops_per_launch = (84 * st["taps"] + 40 * st["energy_evals"] + 84 * st["temporal_taps"]) / n_launch
    bytes_per_eval = bytes_per_launch / max(evals_per_launch, 1)
    flops_per_eval = flops_per_launch / max(evals_per_launch, 1)
    avg_launch_s = st["total_ms"] / n_launch / 1000.0
    achieved = alg_bytes_per_launch / avg_launch_s / 1e9
    achieved_done = bytes_per_launch / avg_launch_s / 1e9
    hbm, peak_kind = peaks()
    sm_mhz = (ck or {}).get("sm_mhz") or 1900.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_achieved = flops_per_launch / avg_launch_s / 1e12
    # every level runs the same propagate passes, so the average launch covers
    # the mean level area
    level_px = float(np.mean([(cfg["w"] >> lv) * (cfg["h"] >> lv) for lv in range(p.levels)]))
    traffic = PROPAGATE_DRAM_BYTES_PER_PIXEL * level_px
    kernel_share = st["total_ms"] / max(sum(v["total_ms"] for v in stats.values()), 1e-9)

    value = dist.ws * frames * args.steps / (total_ms / 1000.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "frames": frames, "image": "%dx%d" % (cfg["w"], cfg["h"]),
                   "exemplar": "%dx%d" % (cfg["ew"], cfg["eh"]), "patch_radius": r, "levels": p.levels,
                   "iterations": p.iterations, "scheme": "FMBM_RM", "histogram": True,
                   "kernels": "generic" if args.generic_kernels else "tiled",
                   "staging": args.staging,
                   "propagate_warps_per_row": args.propagate_lanes or "autotuned",
                   "filter": args.filter,
                   "parallelism": "replicas" if dist.ws > 1 else "single",
                   "l2": "inputs larger than L2 (%.1f GB of resident frame pyramids per step)"
                         % (s.device_bytes / 1e9)},
        "e2e": ({"value": dist.ws * frames * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
                 "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)} if e2e_ms else None),
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "propagate",
                     "bytes": "algorithmic: (32 K + 16) B per evaluation + 32 K B per temporal one, K = %d" % K,
                     "alg_bytes_per_eval": alg_bytes_per_launch / max(evals_per_launch, 1),
                     "work_done": {"achieved": achieved_done, "bytes_per_eval": bytes_per_eval,
                                   "what": "bytes of the taps actually evaluated (early exit, change tracking)"},
                     "l2_gather": {"peak_random_gbs": gc.get("random"), "peak_coherent_gbs": gc.get("coherent"),
                                   "frac_random": achieved / gc["random"] if gc.get("random") else None,
                                   "frac_coherent": achieved / gc["coherent"] if gc.get("coherent") else None,
                                   "what": "32-byte record gathers from an L2-resident 32 MiB buffer, measured "
                                           "here (pt_measure_gather)"},
                     "bytes_per_eval": bytes_per_eval,
                     "temporal_tap_fraction": st["temporal_taps"] / max(st["taps"], 1),
                     "evals_per_launch": evals_per_launch, "avg_launch_ms": avg_launch_s * 1000.0,
                     "time_share": kernel_share,
                     "fp32": {"achieved_tflops": fp32_achieved, "peak_tflops": fp32_peak,
                              "frac": fp32_achieved / fp32_peak, "flops_per_eval": flops_per_eval,
                              "peak_kind": "nominal 152 SM x 128 lanes x 2 at the sampled SM clock"}},
        "kernels": {name: stats[k] for k, name in enumerate(["propagate", "scatter", "residual", "canvas"])},
    }
    if ck:
        line["clocks"] = ck
    if dist.rank == 0 and dist.ws == 1 and not args.no_cpu_baseline:
        act = active_pixels(clip, p.levels, p.distTransCull)
        per_frame = evals_per_step(p, cfg, act, frames) / frames
        counted = sum(v["energy_evals"] for v in stats.values()) / (frames * args.steps)
        threads = os.cpu_count() or 1
        rate, desc, _ = cpu_sample(cfg, p, ex, clip, threads)
        rate1, desc1, _ = cpu_sample(cfg, p, ex, clip, 1)
        line["cpu_baseline"] = {"value": rate / per_frame, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": desc + "; frames/s = evaluations/s / evaluations per frame",
                                "evals_per_s": rate, "extrapolated": True,
                                "single_core": {"value": rate1 / per_frame, "unit": UNIT, "cores": 1,
                                                "evals_per_s": rate1, "sample": desc1}}
        line["evals_per_frame"] = {"schedule": per_frame, "counted": counted}
    s.close()
    if dist.rank == 0 and dist.ws == 1 and not args.no_ref_kernels:
        line["ref_kernels_gpu"] = ref_kernels_gpu(2)
    if dist.rank == 0 and dist.ws == 1 and args.batch_stills > 0:
        line["batched"] = run_batched(args.batch_stills, args.batch_in_flight)
    if dist.rank == 0 and dist.ws == 1 and args.serving_window > 0:
        line["serving"] = run_serving(args.batch_in_flight, args.serving_window, args.serving_budget_gb)
    if dist.rank == 0:
        print(json.dumps(line))
    return 0


def _input_pool():
    """Worker processes (spawned: no CUDA state is inherited) that generate
    the synthetic request inputs in parallel on the host cores."""
    import concurrent.futures
    import multiprocessing
    return concurrent.futures.ProcessPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)),
                                                  mp_context=multiprocessing.get_context("spawn"))


def _exemplar_job(size, seed):
    return synthetic.make_exemplar(size, size, seed=seed)


def _still_job(w, h, seed):
    return synthetic.make_still(w, h, 3, seed=seed)


def _clip_job(w, h, n, seed):
    return synthetic.make_clip(w, h, 3, n, seed=seed)


def _pinned(d):
    """A copy of a dict of arrays in page-locked memory (where a client keeps
    its request data)."""
    from painttween_gb300 import host_array
    out = {}
    for key, v in d.items():
        if isinstance(v, np.ndarray):
            out[key] = host_array(v.shape, v.dtype)
            out[key][...] = v
        else:
            out[key] = v
    return out


def batch_requests(n, seed=7):
    """n independent stills with sizes drawn uniformly from 128x128 to
    1024x1024, each with its own exemplar of a size drawn uniformly from 256
    to 1024 px (the configuration-0 generator), synthesised with the
    configuration-0 settings: patch radius 2, 3 levels, 4 iterations.
    Inputs are in page-locked host memory."""
    rng = np.random.default_rng(seed)
    dims = [tuple(int(v) for v in rng.integers(128, 1025, size=2)) for _ in range(n)]
    esz = [int(v) for v in rng.integers(256, 1025, size=n)]
    with _input_pool() as pool:
        exs = pool.map(_exemplar_job, esz, [100 + i for i in range(n)])
        sts = pool.map(_still_job, [d[0] for d in dims], [d[1] for d in dims], [1000 + i for i in range(n)])
        exs, sts = list(exs), list(sts)
    reqs = []
    for i in range(n):
        p = synthetic.config("still256")["params"]
        reqs.append(dict(params=p, style=_pinned(exs[i]), frames=[_pinned(sts[i])]))
    return reqs


def _latencies(res):
    arr = np.array([r["arrival_ms"] for r in res])
    done = np.array([r["done_ms"] for r in res])
    start = np.array([r["start_ms"] for r in res])
    lat = done - arr
    return {"requests": len(res), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "service_p50_ms": float(np.percentile(done - start, 50)),
            "service_p99_ms": float(np.percentile(done - start, 99)),
            "requests_per_s": len(res) / (max(done.max() - arr.min(), 1e-6) / 1000.0),
            "wall_s": float(done.max() - arr.min()) / 1000.0}


def run_batched(n, in_flight):
    """Batched vs plain on the same GPU: the same requests, all arriving at
    once, through a server (pt_server) one at a time and `in_flight` at a
    time, each after a warm-up run of the same requests.  Latency is from
    arrival to the request's results written in host memory; the service
    time (admission to results) is kept beside it.  The single-request
    latency is each request's service time on the plain path."""
    from painttween_gb300.serving import Server
    reqs = batch_requests(n)
    out = {"workload": "%d stills 128-1024 px, each with its own exemplar of 256-1024 px, r2 / 3 levels / 4 "
                       "iterations, all arriving at once" % n,
           "latency": "arrival to results in host memory, ms"}
    for name, k in (("plain", 1), ("batched", in_flight)):
        with Server(max_in_flight=k) as srv:
            srv.run(reqs, offsets=False, pinned=True)  # warm-up: the workers' contexts and memory caches
            res = srv.run(reqs, offsets=False, pinned=True)
        out[name] = dict(_latencies(res), in_flight=k)
    out["speedup"] = out["batched"]["requests_per_s"] / out["plain"]["requests_per_s"]
    out["p99_vs_single"] = out["batched"]["p99_ms"] / out["plain"]["service_p50_ms"]
    # the summed durations of the requests' patch-distance and canvas
    # launches, request by request on one context (per-launch CUDA events):
    # small requests' launches leave most SMs idle, so overlapping requests
    # finishes faster than this serial kernel time
    from painttween_gb300 import Synthesizer
    s = Synthesizer(device=0)
    busy_ms = 0.0
    try:
        for rq in reqs:
            fr, st = rq["frames"][0], rq["style"]
            h, w = fr["rgba"].shape[:2]
            s.setup(rq["params"], w, h, st["w"], st["h"], 1)
            s.set_style(0, st["base"], st["output"], st["orient_tensor"], st["dist_trans"], st["object_ids"])
            s.set_frame_dict(0, fr)
            s.set_profiling(_abi.PROFILE_TIMING)
            s.synthesize_frame(0)
            busy_ms += sum(s.kernel_stats(k)["total_ms"] for k in range(4))
            s.set_profiling(0)
    finally:
        s.close()
    out["serial_kernel_s"] = busy_ms / 1000.0
    out["batched"]["wall_vs_serial_kernels"] = out["batched"]["wall_s"] / out["serial_kernel_s"]
    return out


def serving_requests(n, seed, clip_pool):
    """n requests of the serving mix: 70 % stills of 128-1024 px (the
    configuration-0 settings) and 30 % clips of 8-24 frames (the
    configuration-1 settings: radius 2, 4 levels, 4 iterations, temporal
    coherence 0.5), each with its own exemplar of 256-1024 px.  A clip is the
    first frames of one of `clip_pool`'s 24-frame clips (512x512 to
    1920x1080, the configuration-1 motion)."""
    rng = np.random.default_rng(seed)
    kinds = rng.random(n) < 0.7
    esz = [int(v) for v in rng.integers(256, 1025, size=n)]
    dims = [tuple(int(v) for v in rng.integers(128, 1025, size=2)) for _ in range(n)]
    which = [int(v) for v in rng.integers(0, len(clip_pool), size=n)]
    nfr = [int(v) for v in rng.integers(8, 25, size=n)]
    stills = [i for i in range(n) if kinds[i]]
    with _input_pool() as pool:
        exs = list(pool.map(_exemplar_job, esz, [5000 + seed * 1000 + i for i in range(n)]))
        sts = list(pool.map(_still_job, [dims[i][0] for i in stills], [dims[i][1] for i in stills],
                            [7000 + seed * 1000 + i for i in stills]))
    sts = dict(zip(stills, sts))
    reqs = []
    for i in range(n):
        if kinds[i]:
            p = synthetic.config("still256")["params"]
            frames = [_pinned(sts[i])]
        else:
            p = synthetic.config("anim512")["params"]
            frames = clip_pool[which[i]][:nfr[i]]
        reqs.append(dict(params=p, style=_pinned(exs[i]), frames=frames, kind="still" if kinds[i] else "clip"))
    return reqs


def run_serving(in_flight, window_s, budget_gb, seed=11):
    """The serving mix on one GPU.  (1) Capacity: a set of requests arriving
    at once, through the plain path (one at a time) and the server
    (`in_flight` at a time).  (2) Poisson arrivals over a window of
    `window_s` seconds at 80 % of the server's capacity and at the nominal
    100 requests/s, each run until its queue has drained; latency from
    arrival, sustained requests/s over the run, and whether the queue stayed
    bounded (the last quarter's latencies no more than twice the first
    quarter's)."""
    from painttween_gb300.serving import Server
    sizes = [(512, 512), (960, 540), (1280, 720), (1920, 1080)]
    with _input_pool() as pool:
        clips = list(pool.map(_clip_job, [s[0] for s in sizes], [s[1] for s in sizes], [24] * len(sizes),
                              [9000 + k for k in range(len(sizes))]))
    clip_pool = [[_pinned(fr) for fr in c] for c in clips]
    del clips
    budget = int(budget_gb * 1e9)
    out = {"mix": "70 % stills 128-1024 px (r2, 3 levels, 4 iterations), 30 % clips of 8-24 frames of "
                  "512x512 / 960x540 / 1280x720 / 1920x1080 (r2, 4 levels, 4 iterations, temporal 0.5, "
                  "forward + backward passes); each request with its own exemplar of 256-1024 px",
           "budget_gb": budget_gb, "in_flight": in_flight,
           "latency": "arrival to results in host memory, ms"}
    cap_reqs = serving_requests(20, seed, clip_pool)
    for name, k in (("plain", 1), ("server", in_flight)):
        with Server(max_in_flight=k, hbm_budget=budget) as srv:
            srv.run(cap_reqs[:6], offsets=False, pinned=True)  # warm-up
            res = srv.run(cap_reqs, offsets=False, pinned=True)
        out["capacity_" + name] = _latencies(res)
    cap = out["capacity_server"]["requests_per_s"]
    out["capacity_speedup"] = cap / out["capacity_plain"]["requests_per_s"]
    rng = np.random.default_rng(seed + 1)
    runs = []
    # the nominal rate's window is cut to 50 arrivals, so that its backlog
    # drains within the run
    for rate, win in ((0.8 * cap, window_s), (100.0, min(window_s, 0.5))):
        n = max(4, int(round(rate * win)))
        reqs = serving_requests(n, seed + 2 + len(runs), clip_pool)
        t = np.cumsum(rng.exponential(1000.0 / rate, size=n))
        for r, a in zip(reqs, t):
            r["arrival_ms"] = float(a)
        with Server(max_in_flight=in_flight, hbm_budget=budget) as srv:
            srv.run(cap_reqs[:6], offsets=False, pinned=True)  # warm-up
            res = srv.run(reqs, offsets=False, pinned=True)
        lat = np.array([r["latency_ms"] for r in res])
        q = max(1, n // 4)
        bounded = bool(np.mean(lat[-q:]) <= 2.0 * np.mean(lat[:q]))
        st = _latencies(res)
        still_lat = [r["latency_ms"] for r, rq in zip(res, reqs) if rq["kind"] == "still"]
        st.update(arrival_rate=rate, window_s=float(t[-1] / 1000.0), bounded=bounded,
                  still_p50_ms=float(np.percentile(still_lat, 50)) if still_lat else None,
                  peak_context_gb=max(r["device_bytes"] for r in res) / 1e9)
        runs.append(st)
    out["poisson"] = runs
    ok = [r["arrival_rate"] for r in runs if r["bounded"]]
    out["max_bounded_rate"] = max(ok) if ok else None
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frames", type=int, default=0, help="override the clip length (testing only)")
    ap.add_argument("--e2e-steps", type=int, default=-1, help="end-to-end steps (default: as many as --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-kernels", action="store_true", help="skip timing the reference's kernels on the GPU")
    ap.add_argument("--batch-stills", type=int, default=64, help="requests of the batched-vs-plain run (0: skip)")
    ap.add_argument("--batch-in-flight", type=int, default=8)
    ap.add_argument("--serving-window", type=float, default=8.0,
                    help="seconds of Poisson arrivals per rate of the serving run (0: skip)")
    ap.add_argument("--serving-budget-gb", type=float, default=150.0)
    ap.add_argument("--filter", default="texture", choices=["texture", "exact"],
                    help="bilinear arithmetic: the texture unit's (the reference's) or exact FP32")
    ap.add_argument("--staging", default="tma", choices=["tma", "loads"],
                    help="how the tiled kernels stage interior tiles: tensor copies or plain loads (same results)")
    ap.add_argument("--propagate-lanes", type=int, default=0, choices=[0, 1, 2],
                    help="propagate's warps per tile row: 0 = autotuned per launch shape (same results)")
    ap.add_argument("--generic-kernels", action="store_true",
                    help="run the generic one-thread-per-pixel kernels instead of the tiled ones (profiling only)")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        return run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
