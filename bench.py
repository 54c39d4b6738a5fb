#!/usr/bin/env python3
"""Benchmark of the renderer core: path-traced Mpx*spp/s on the config-1 scene.

Workload (default): 256 UV spheres (64x32 segments, 1,015,808 triangles) +
a 40x40 ground quad, 50/50 matte / physically-based materials, one
directional light (irradiance 3), ambient 0.2, 1024x1024, 64 samples per
pixel per frame, maximum depth 5; BVH built on the device at commit. One
step = one frame (64 spp over every pixel) rendered through the C ABI.

  value : W*H*spp / render-kernel time (CUDA events on the render stream),
          scene resident in HBM, L2 flushed (256 MiB write) between steps.
  e2e   : the same metric through the public call sequence with host
          buffers: camera update + commit, render, wait, map the colour,
          depth, normal and albedo channels into host memory (wall clock).

--impl reference times the CPU restatement of the reference CPU device
(the oracle, 64x64 tiles on all host threads) on a bounded band of rows of
the same workload; there is no runnable reference binary in this
environment (Visionaray and the ANARI SDK are not available).
"""
import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MPX = 1e6


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--res", type=int, default=1024)
    p.add_argument("--spp", type=int, default=64)
    p.add_argument("--e2e-steps", type=int, default=8)
    p.add_argument("--cpu-rows", type=int, default=192,
                   help="rows of the frame the CPU baseline renders (bounded sample)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--accum-frames", type=int, default=64,
                   help="config 1 also as this many accumulated 1-spp frames (0: skip)")
    p.add_argument("--bvh-leaf-size", type=int, default=None,
                   help="world parameter bvhLeafSize of the config-1 and -2 scenes (default: the library's)")
    p.add_argument("--sample-chunks", type=int, default=16,
                   help="config 1: the frame's samples as this many concurrent per-pixel streams "
                        "(accumulated sub-frames); 1 = one stream per pixel and frame")
    p.add_argument("--wavefront", action="store_true",
                   help="path tracer with wavefront queues instead of one thread per pixel")
    p.add_argument("--no-raycast", dest="raycast", action="store_false",
                   help="skip the config-0 raycast (volume marcher) measurement")
    p.add_argument("--no-volume", dest="volume", action="store_false",
                   help="skip the config-2 volumetric path-tracing measurement")
    p.add_argument("--volume-res", type=int, nargs=2, default=[1920, 1080],
                   help="config-2 frame size (full size by default; smaller for profiling)")
    p.add_argument("--volume-spp", type=int, default=256)
    p.add_argument("--volume-sample-chunks", type=int, default=8,
                   help="config 2: the frame's samples as this many per-pixel streams")
    p.add_argument("--no-denoise", dest="denoise", action="store_false",
                   help="skip the config-4 denoiser training and evaluation")
    p.add_argument("--denoise-train-scenes", type=int, default=128)
    p.add_argument("--denoise-eval-scenes", type=int, default=8)
    p.add_argument("--denoise-steps", type=int, default=4000)
    p.add_argument("--denoise-forward-only", action="store_true",
                   help="config 4: time only the 1080p denoiser pass (untrained weights), "
                        "no data, training or evaluation")
    p.add_argument("--no-batch", dest="batch", action="store_false",
                   help="skip the config-3 batched-rendering measurement")
    p.add_argument("--batch-only", action="store_true",
                   help="profiling aid: run only the config-3 measurement and print its record "
                        "(no config-1 metric line); its second sequential pass is bracketed by "
                        "cudaProfilerStart/Stop for ncu --profile-from-start off")
    return p.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def measured_peaks_tensor(sustained=False):
    """bf16 tensor peak in TFLOP/s: the burst figure (a kernel timed alone)
    or the sustained one (a kernel timed inside a long loop)."""
    key = "bf16_tflops_sustained" if sustained else "bf16_tflops"
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        if key in d:
            return d[key], "measured"
    return (1700.0 if sustained else 1900.0), "fallback"


def profiled_value(name, key):
    """A 'key = value' line's value from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for ln in f:
            if ln.strip().startswith(key + " "):
                try:
                    return float(ln.split("=")[1].split()[0])
                except (IndexError, ValueError):
                    return None
    return None


def profiled_traffic(name="pathtrace_config1.txt"):
    """DRAM bytes per launch (per frame) from a committed ncu summary."""
    return profiled_value(name, "traffic_bytes_per_launch")


def profiled_metric(name, metric):
    """A metric's value from a committed ncu summary line '<metric>  <value> ...'."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for ln in f:
            parts = ln.split()
            if len(parts) >= 2 and parts[0] == metric:
                try:
                    return float(parts[1])
                except ValueError:
                    return None
    return None


def cpu_baseline(scene, rows, threads=0, keep=False):
    """Time the oracle on a band of rows spread over the frame; Mpx*spp/s.
    keep: also return the row ranges and the oracle's colour image."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    S = po.Scene(scene)
    W, H = scene["frame"]["size"]
    spp = scene["renderer"]["pixelSamples"]
    F = po.Frame(W, H)
    bands = 8
    per = max(1, rows // bands)
    starts = [int((b + 0.5) * H / bands) - per // 2 for b in range(bands)]
    t0 = time.perf_counter()
    for s in starts:
        po.render(S, F, num_threads=threads, rows=(s, s + per))
        F.f.accumID = 0  # every band is the frame's first (the row ranges are disjoint)
    dt = time.perf_counter() - t0
    px = W * per * bands
    cores = threads if threads > 0 else os.cpu_count()
    if keep:
        return px * spp / dt / MPX, dt, px, cores, [(s, s + per) for s in starts], F.color
    return px * spp / dt / MPX, dt, px, cores


def phase_split(c):
    """From the counting frame's statistics: the share of the path tracer's
    per-thread time spent in surface traversal and in delta tracking, and
    the SIMT efficiency (active lanes / 32) of the traversal's inner-node
    and leaf loops."""
    if len(c) < 30 or not c[24]:
        return {}
    out = {"time_share_surface_traversal": c[25] / c[24],
           "time_share_delta_tracking": c[26] / c[24]}
    if c[27]:
        out["simt_inner_node_loop"] = c[1] / (32.0 * c[27] / 65536.0)
    if c[29]:
        out["simt_leaf_loop"] = c[28] / (32.0 * c[29] / 65536.0)
    return out


def issue_roofline(kernel_s, spp, res, sms=None):
    """The path tracer's issue roofline: thread instructions per second of
    the frame (warp instructions x active lanes per warp instruction of the
    profiled launch at the same resolution, scaled by spp over the profiled
    launch's spp, over the live kernel time) against the SMs' peak (SMs x 4
    schedulers x 32 lanes x the maximum SM clock): frac = issue rate x SIMT
    efficiency."""
    inst = profiled_metric("pathtrace_config1.txt", "smsp__inst_executed.sum")
    pspp = profiled_value("pathtrace_config1.txt", "profiled_spp_per_launch") or 1.0
    lanes = profiled_metric("pathtrace_config1.txt",
                            "smsp__thread_inst_executed_per_inst_executed.ratio")
    active = profiled_metric("pathtrace_config1.txt",
                             "smsp__issue_active.avg.pct_of_peak_sustained_active")
    if not inst or not lanes or res != 1024:
        return None
    if sms is None:
        import torch

        sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = 2070.0
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            mhz = json.load(f).get("sm_max_mhz", mhz)
    peak = sms * 4 * 32 * mhz * 1e6 / 1e9
    achieved = inst * lanes * (spp / pspp) / kernel_s / 1e9
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Gthread-inst/s",
            "frac": achieved / peak,
            "issue_active_frac": active / 100 if active is not None else None,
            "active_lanes_per_warp_instruction": lanes,
            "note": f"thread instructions of the profiled {pspp:.0f}-spp launch ({inst:.4g} warp "
                    f"instructions x {lanes:.2f} lanes) x {spp}/{pspp:.0f} / live kernel time, against "
                    f"{sms} SMs x 4 schedulers x 32 lanes x {mhz:.0f} MHz; frac = issue-active "
                    "share x SIMT efficiency"}


def measure_l2_read_peak(pkg, mib=8, repeats=64, trials=5):
    """Achievable L2 read bandwidth on this GPU, measured in this run: a
    streaming read (16-byte L2-only loads, every SM) of a `mib` MiB buffer
    (config 0's field is 8 MiB) `repeats` times per launch, timed with CUDA
    events on torch's current stream (the one the read is launched on);
    best of `trials` launches. GB/s."""
    import ctypes
    import torch

    probe = ctypes.CDLL(os.path.join(os.path.dirname(pkg.__file__), "libvsr_probe.so"))
    probe.vsrProbeReadBandwidth.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    nbytes = mib << 20
    buf = torch.ones(nbytes // 4, dtype=torch.float32, device="cuda")
    blocks = 4
    sink = torch.zeros(torch.cuda.get_device_properties(0).multi_processor_count * blocks,
                       dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    best = 0.0
    for t in range(trials + 1):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        rc = probe.vsrProbeReadBandwidth(buf.data_ptr(), nbytes, repeats, blocks,
                                         sink.data_ptr(), stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        if rc:
            return None
        if t > 0:  # the first launch is a warm-up
            best = max(best, nbytes * repeats / (a.elapsed_time(b) * 1e-3) / 1e9)
    return {"gbs": best, "buffer_mib": mib, "repeats": repeats,
            "how": "streaming 16-byte ld.global.cg reads over every SM, CUDA events, best of "
                   f"{trials}"}


def measure_raycast_config0(pkg, dev, flush, steps=20, gradient=False, l2=None):
    """Config 0 (raycast, 128^3 blob volume, 512x512, 1 spp): Mpx/s and the
    marcher's roofline (32 B per trilinear sample + 20 B per pixel written).
    gradient: the same volume lit by a directional light with gradient
    shading (6 more trilinear samples per step for the central differences:
    7 x 32 B per step)."""
    import torch

    scene = pkg.scenes.config0()
    fetches = 1
    if gradient:
        scene["lights"] = [{"direction": [-0.3, -0.87, -0.39], "color": [1.0, 1.0, 1.0],
                            "irradiance": 2.5}]
        scene["renderer"]["gradientShading"] = True
        fetches = 7
    h = pkg.scenes.build(dev, scene, channels=("color", "depth"))
    frame = h["frame"]
    dev.set(frame, "collectStatistics", True)
    dev.commit(frame)
    dev.render(frame)
    dev.wait(frame)
    samples = (dev.get_u64(frame, "statistics", 8) or [0] * 8)[3]
    dev.set(frame, "collectStatistics", False)
    dev.commit(frame)
    for _ in range(3):
        dev.render(frame)
        dev.wait(frame)
    ds = []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        dev.render(frame)
        dev.wait(frame)
        ds.append(dev.get_float(frame, "duration.render"))
    t = statistics.mean(ds)
    W, H = scene["frame"]["size"]
    alg = samples * 32 * fetches + W * H * 20
    peak, kind = measured_peaks()
    for o in (frame, h["renderer"], h["camera"], h["world"], *h["keep"]):
        dev.release(o)
    if gradient:
        return {"value": W * H / t / MPX, "unit": "Mpx*spp/s", "ms_per_frame": 1e3 * t,
                "workload": "config0 volume with a directional light and gradient shading, "
                            "512x512 1spp, per-pixel raycast kernel",
                "march_samples": samples,
                "roofline": {"bound": "hbm", "achieved": alg / t / 1e9, "peak": peak,
                             "unit": "GB/s", "frac": alg / t / 1e9 / peak, "traffic": None,
                             "note": f"7 x 32 B per step (the sample and its 6 central "
                                     f"differences) + 20 B per pixel; peak {kind}"}}
    achieved = alg / t / 1e9
    l2_roof = None
    if l2:
        l2_roof = {"bound": "l2", "achieved": achieved, "peak": l2["gbs"], "unit": "GB/s",
                   "frac": achieved / l2["gbs"],
                   "note": f"the same algorithmic bytes against the L2 read bandwidth "
                           f"measured in this run ({l2['buffer_mib']} MiB buffer; the field "
                           f"is L2-resident)"}
    return {"value": W * H / t / MPX, "unit": "Mpx*spp/s", "ms_per_frame": 1e3 * t,
            "workload": "config0 raycast 512x512 1spp, 128^3 float32 blobs, dt 0.5 voxel",
            "march_samples": samples,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": profiled_traffic("raycast_config0.txt"),
                         "note": f"32 B per trilinear sample + 20 B per pixel; peak {kind}; "
                                 "segmented marcher (set-up, 12-sample segments, combine; passes launched as programmatic dependents); "
                                 "the 8 MiB field is L2-resident, so DRAM traffic is far "
                                 "below the algorithmic bytes"},
            "roofline_l2": l2_roof}


def measure_batch_config3(pkg, dev, steps=3, num_scenes=64, profile_range=False):
    """Config 3 (64 independent scenes: blob volumes of side 64..384, optional
    10k..500k-triangle sphere sets, images 256^2..1024^2, 1..64 spp, raycast
    and path tracing): the 64 frames as one batch (vsrRenderFrames, CUDA
    graph, tuned tiles) against the same frames rendered one after another
    with vsrRenderFrame. Both are timed on the host from the first call to
    the end of the last frame; each step renders every frame once more."""
    t_gen = time.perf_counter()
    scenes = pkg.scenes.config3(num_scenes=num_scenes)
    gen_s = time.perf_counter() - t_gen
    hs = [pkg.scenes.build(dev, sc, channels=("color", "depth")) for sc in scenes]
    frames = [h["frame"] for h in hs]
    # the raycast renderer takes one sample per pixel (pixelSamples is a
    # path-tracer parameter)
    px_spp = sum(sc["frame"]["size"][0] * sc["frame"]["size"][1] *
                 (sc["renderer"]["pixelSamples"] if sc["renderer"]["type"] == "pathtrace" else 1)
                 for sc in scenes)

    def wait_all():
        for f in frames:
            dev.wait(f)

    def sequential():
        t = time.perf_counter()
        for f in frames:
            dev.render(f)
        wait_all()
        return time.perf_counter() - t

    def batched():
        t = time.perf_counter()
        dev.render_batch(frames)
        wait_all()
        return time.perf_counter() - t

    sequential()  # commits, BVH builds, first-use allocations
    # what caps batching: each frame's own device time in a sequential pass
    # (the share of it with idle SMs comes from the committed profile)
    if profile_range:
        import torch

        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStart()
    sequential()
    if profile_range:
        torch.cuda.cudart().cudaProfilerStop()
    per = []
    for sc, f in zip(scenes, frames):
        W, H = sc["frame"]["size"]
        spp = sc["renderer"]["pixelSamples"] if sc["renderer"]["type"] == "pathtrace" else 1
        per.append((sc["renderer"]["type"], W * H * spp, dev.get_float(f, "duration.render")))
    t_seq_dev = sum(t for _, _, t in per)
    tune = 0
    while not dev.get_int(frames[0], "batch.tuned") and tune < 32:
        batched()
        tune += 1
    batched()
    seq = [sequential() for _ in range(steps)]
    bat = [batched() for _ in range(steps)]
    err = 0
    for f in frames:
        err |= dev.get_uint(f, "errorFlags") or 0
    tile_w, fetch = dev.get_int(frames[0], "batch.tileWidth"), dev.get_int(frames[0], "batch.fetch")
    for h in hs:
        for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
            dev.release(o)
    ts, tb = statistics.mean(seq), statistics.mean(bat)
    kinds = {k: sum(1 for sc in scenes if sc["renderer"]["type"] == k) for k in ("raycast", "pathtrace")}
    return {"value": px_spp / tb / MPX, "unit": "Mpx*spp/s", "batched_ms": 1e3 * tb,
            "sequential_ms": 1e3 * ts, "speedup_vs_sequential": ts / tb,
            "sequential_value": px_spp / ts / MPX,
            "workload": f"config3 {num_scenes} scenes ({kinds['raycast']} raycast, "
                        f"{kinds['pathtrace']} pathtrace), {px_spp / 1e6:.0f} Mpx*spp per pass",
            "tile": f"{tile_w}x{32 // max(tile_w, 1)}", "fetch": fetch, "tuning_batches": tune,
            "error_flags": err, "generate_s": gen_s,
            "cap_analysis": {
                "sum_frame_device_ms": 1e3 * t_seq_dev,
                "sm_active_share": profiled_value("batch_config3.txt", "sm_active_share"),
                "max_speedup_from_filling_idle_sms":
                    profiled_value("batch_config3.txt", "max_speedup_from_filling_idle_sms"),
                "how": "each frame's device time in a sequential pass (measured here); the share of "
                       "that pass in which the SMs were active, time-weighted over its launches "
                       "(ncu, profiles/batch_config3.txt): a batch can only fill the idle rest"},
            "timing": "host wall clock, first call to last frame done; synthetic seeded scenes"}


def time_denoiser_1080p(dev, dn, D, masked_out=None):
    """At 1920x1080: path-tracing seconds per sample per pixel, and the
    median seconds of one denoiser pass (vsrDenoiseFrame: input assembly,
    network, gate) after 3 warm-up passes, as host wall time (with the
    launches and the synchronisation of the call) and as device time (CUDA
    events on the device's stream)."""
    import torch

    sc = D.training_scene(10001, res=1920, spp=16)
    sc["frame"]["size"] = (1920, 1080)
    sc["camera"]["aspect"] = 1920 / 1080
    h = D.build(dev, sc, variance=True)
    for _ in range(2):
        dev.render(h["frame"])
        dev.wait(h["frame"])
    pt = []
    for _ in range(3):
        dev.render(h["frame"])
        dev.wait(h["frame"])
        pt.append(dev.get_float(h["frame"], "duration.render"))
    pt_s_per_spp = statistics.median(pt) / 16
    out = torch.zeros((1920 * 1080, 4), dtype=torch.float32, device="cuda")
    for _ in range(3):
        dn.denoise_frame(h["frame"], out.data_ptr())
    ds = []
    stream = torch.cuda.ExternalStream(dev.lib.vsrDeviceStream(dev.handle))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    dev_ms = []
    for _ in range(10):
        tt = time.perf_counter()
        ev[0].record(stream)
        dn.denoise_frame(h["frame"], out.data_ptr())  # synchronous: returns the retry count
        ev[1].record(stream)
        ds.append(time.perf_counter() - tt)
        ev[1].synchronize()
        dev_ms.append(ev[0].elapsed_time(ev[1]))
    # frames restricted to the gate's rejected pixels: device time per
    # rendered pixel-sample (warps with few rejected pixels still cost)
    mask = torch.zeros(1920 * 1080, dtype=torch.uint8, device="cuda")
    nret = dn.denoise_frame(h["frame"], out.data_ptr(), k=3.0, floor=0.01, retry_ptr=mask.data_ptr())
    masked = None
    if nret:
        dev.sample_mask(h["frame"], mask.data_ptr())
        mt = []
        for _ in range(3):
            dev.render(h["frame"])
            dev.wait(h["frame"])
            mt.append(dev.get_float(h["frame"], "duration.render"))
        dev.sample_mask(h["frame"], None)
        masked = {"retry_pixels": nret, "retry_share": nret / (1920 * 1080),
                  "frame_ms": 1e3 * statistics.median(mt),
                  "s_per_px_spp": statistics.median(mt) / (nret * 16)}
    D.release(dev, h)
    if masked_out is not None:
        masked_out.update(masked or {})
    return pt_s_per_spp, statistics.median(ds), 1e-3 * statistics.median(dev_ms)


DENOISER_LAYERS = [(16, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 128, 2), (128, 128, 2),
                   (128, 256, 3), (256, 256, 3), (384, 128, 2), (128, 128, 2), (192, 64, 1),
                   (64, 64, 1), (96, 32, 0), (32, 32, 0), (32, 16, 0)]


def denoiser_roofline(dn_s):
    flops = sum(2.0 * ci * co * 9 * 1920 * 1080 / 4 ** lvl for ci, co, lvl in DENOISER_LAYERS)
    peak = measured_peaks_tensor()
    return {"bound": "tensor", "achieved": flops / dn_s / 1e12, "peak": peak[0],
            "unit": "TFLOP/s", "frac": flops / dn_s / 1e12 / peak[0],
            "note": f"denoiser forward at 1920x1080 ({flops / 1e12:.3f} TFLOP; the device "
                    f"time of the whole pass, CUDA events, with its input and gate kernels); "
                    f"peak bf16 {peak[1]}; "
                    "tcgen05.mma kind::f16 (bf16 -> fp32 in tensor memory), persistent "
                    "warp-specialised kernel (TMA producer, MMA thread, epilogue warps) "
                    "on 4 x 128-pixel halo tiles of channel-blocked activations; "
                    "decoders read upsampled level and skip in place"}


def denoiser_train_roofline(ms_per_step, batch=16, crop=128):
    """Tensor roofline of one training step: the forward pass, the weight
    gradient of every layer and the input gradient of every layer but the
    first (the network's input needs none), each 2 Cin Cout 9 flops per
    pixel of its level, over the measured step time (which also holds the
    loss, pooling, upsampling and Adam kernels), against the sustained bf16
    peak (the step runs in a loop of thousands)."""
    px = batch * crop * crop
    per = [2.0 * ci * co * 9 * px / 4 ** lvl for ci, co, lvl in DENOISER_LAYERS]
    flops = 2 * sum(per) + sum(per[1:])
    peak = measured_peaks_tensor(sustained=True)
    achieved = flops / (ms_per_step * 1e-3) / 1e12
    return {"bound": "tensor", "achieved": achieved, "peak": peak[0], "unit": "TFLOP/s",
            "frac": achieved / peak[0],
            "note": f"training step of {batch} {crop}^2 crops ({flops / 1e9:.1f} GFLOP: forward, "
                    f"weight and input gradients) over the measured step time; peak bf16 "
                    f"sustained {peak[1]}"}


def measure_denoiser_forward(pkg, dev):
    """The 1080p denoiser pass alone (weights as initialised; the time does
    not depend on their values), for profiling the network's kernels."""
    D = importlib.import_module(pkg.__name__ + ".denoise")
    dn = pkg.vsr.Denoiser(dev, seed=1)
    pt_s_per_spp, dn_s, dn_dev_s = time_denoiser_1080p(dev, dn, D)
    dn.close()
    return {"workload": "config4 denoiser forward at 1920x1080 (untrained weights)",
            "pt_ms_per_spp_1080p": 1e3 * pt_s_per_spp, "denoise_ms_1080p": 1e3 * dn_s,
            "denoise_device_ms_1080p": 1e3 * dn_dev_s,
            "roofline": denoiser_roofline(dn_dev_s)}


def measure_denoiser_config4(pkg, dev, train_scenes=128, eval_scenes=8, steps=4000,
                             train_ref_spp=1024, eval_ref_spp=4096, res=256):
    """Config 4 (learned denoiser): train the U-Net on path-traced pairs
    (inputs after 4, 8, 16 and 32 spp, 1024-spp references, 256^2 images,
    128^2 crops, batch 16, L1 on log colour, Adam with cosine decay), then
    on held-out scenes compare plain path tracing (4..256 spp) and denoised
    path tracing against 4096-spp references, and turn the RMSEs into the
    time to reach the plain 256-spp RMSE at 1920x1080 from the measured
    per-sample render time and denoiser time there."""
    import torch

    D = importlib.import_module(pkg.__name__ + ".denoise")
    t0 = time.perf_counter()
    x, t = D.make_dataset(dev, list(range(1, 1 + train_scenes)), res=res, ref_spp=train_ref_spp,
                          input_spp=(4, 8, 16, 32))
    data_s = time.perf_counter() - t0
    dn = pkg.vsr.Denoiser(dev, seed=1)
    losses, train_s = D.train(dn, x, t, steps, lr=2e-3, log_every=max(1, steps // 4))
    del x, t
    levels = (4, 8, 12, 16, 20, 24, 32, 64)  # frames accumulate 4 spp per render
    ev = D.evaluate(dev, dn, list(range(10001, 10001 + eval_scenes)), res=res,
                    ref_spp=eval_ref_spp, denoise_levels=levels)
    masked = {}
    pt_s_per_spp, dn_s, dn_dev_s = time_denoiser_1080p(dev, dn, D, masked_out=masked)
    loop = D.evaluate_gated_loop(dev, dn, list(range(10001, 10001 + eval_scenes)), res=res,
                                 ref_spp=eval_ref_spp)
    dn.close()
    if masked.get("s_per_px_spp"):
        loop = D.gated_loop_times(loop, pt_s_per_spp, dn_s, masked["s_per_px_spp"])
    goal, t_plain, s_dn, t_dn = D.time_to_rmse(ev["plain"]["rmse_tm"], ev["denoised"]["rmse_tm"],
                                               pt_s_per_spp, dn_s)
    four = D.at_input_spp(ev["plain"]["rmse_tm"], ev["denoised"]["rmse_tm"], pt_s_per_spp, dn_s, 4)
    four["reaches_plain256_rmse"] = four["denoised_rmse_tm"] <= goal
    return {
        "workload": f"config4 denoiser: {train_scenes} training scenes x 4 input spp levels "
                    f"({res}^2, {train_ref_spp}-spp references), {steps} Adam steps of 16 "
                    f"128^2 crops; {eval_scenes} held-out scenes vs {eval_ref_spp}-spp references",
        "plain": ev["plain"], "denoised": ev["denoised"], "gated": ev["gated"],
        "gate_retry_share": ev["retry"],
        "error_measure": "RMSE of Reinhard tone-mapped colour c/(1+c) against the reference "
                         "(linear RMSE reported too; it is dominated by rare very bright samples)",
        "goal_rmse_tm_plain256": goal, "plain256_s_1080p": t_plain,
        "denoised_input_spp": s_dn, "denoised_s_1080p": t_dn,
        "speedup_to_equal_rmse": (t_plain / t_dn) if t_dn else None,
        "at_4_input_spp": four,
        "gated_loop": {
            "rounds": loop, "masked_frames_1080p": masked,
            "reaches_goal_at_round": next((e["round"] for e in loop if e["rmse_tm"] <= goal), None),
            "speedup_to_goal": next((t_plain / e["s_1080p"] for e in loop
                                     if e["rmse_tm"] <= goal and "s_1080p" in e), None),
            "how": "4 input spp, denoise + variance gate (k 3, floor 0.01); rejected pixels get "
                   "4 more frames of 4 spp through the frame's sample mask per round; seconds "
                   "at 1080p from the measured per-sample, masked per-pixel-sample and denoiser "
                   "times"},
        "pt_ms_per_spp_1080p": 1e3 * pt_s_per_spp, "denoise_ms_1080p": 1e3 * dn_s,
        "denoise_device_ms_1080p": 1e3 * dn_dev_s,
        "train_s": train_s, "train_ms_per_step": 1e3 * train_s / steps, "data_s": data_s,
        "train_roofline": denoiser_train_roofline(1e3 * train_s / steps),
        "loss": losses,
        "roofline": denoiser_roofline(dn_dev_s),
    }


def measure_volume_config2(pkg, dev, flush, count_spp=8, res=(1920, 1080), spp=256, chunks=8,
                           leaf_size=None):
    """Config 2 (volumetric path tracing, 512^3 value noise with 16^3-voxel
    brick majorants + the config-1 spheres, 1920x1080, 256 spp, depth 8,
    clip plane): Mpx*spp/s of one full frame, and the delta-tracking
    roofline from a counting frame at count_spp samples scaled to 256."""
    import torch

    scene = pkg.scenes.config2(res=tuple(res), spp=spp)
    # the frame's samples as concurrent per-pixel streams (sample chunks:
    # the sub-frames the reference accumulates over that many frames); 8
    # are 3 % faster than one stream per pixel
    scene["renderer"]["sampleChunks"] = chunks
    if leaf_size is not None:
        scene["bvhLeafSize"] = leaf_size
    W, H = scene["frame"]["size"]
    count_spp = min(count_spp, spp)
    spp = scene["renderer"]["pixelSamples"]
    h = pkg.scenes.build(dev, scene, channels=("color", "depth"))
    frame, rend = h["frame"], h["renderer"]
    dev.render(frame)  # BVH build + warm-up
    dev.wait(frame)
    flush.fill_(1.0)
    torch.cuda.synchronize()
    dev.render(frame)
    dev.wait(frame)
    t = dev.get_float(frame, "duration.render")
    err = dev.get_uint(frame, "errorFlags")
    dev.set(rend, "pixelSamples", count_spp)
    dev.set(rend, "sampleChunks", 1)
    dev.commit(rend)
    dev.set(frame, "collectStatistics", True)
    dev.commit(frame)
    dev.render(frame)
    dev.wait(frame)
    c = dev.get_u64(frame, "statistics", 24) or [0] * 24
    scale = spp / count_spp
    track, cells = c[4] * scale, c[5] * scale
    alg = track * 32 + cells * 4 + W * H * 20
    peak, kind = measured_peaks()
    for o in (frame, rend, h["camera"], h["world"], *h["keep"]):
        dev.release(o)
    return {"value": W * H * spp / t / MPX, "unit": "Mpx*spp/s", "ms_per_frame": 1e3 * t,
            "workload": f"config2 volumetric pathtracer {W}x{H} {spp}spp depth8, 512^3 value noise "
                        "(16^3 bricks) + 1015810 tris, clip plane",
            "sample_chunks": chunks,
            "error_flags": err,
            "tracking_samples_est": track, "majorant_cells_est": cells,
            "roofline": {"bound": "hbm", "achieved": alg / t / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / t / 1e9 / peak,
                         "note": f"delta tracking only: 32 B per tentative collision + 4 B per "
                                 f"brick + frame bytes, counts from a {count_spp}-spp frame scaled "
                                 f"to {spp} spp; peak {kind}"}}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    pkg = importlib.import_module("anari-visionaray_gb300")
    scene = pkg.scenes.config1(res=args.res, spp=args.spp)
    rows = max(8, args.cpu_rows // 2)
    vals = []
    for i in range(args.warmup + args.steps):
        v, dt, px, cores = cpu_baseline(scene, rows)
        if i >= args.warmup:
            vals.append((v, dt))
    value = sum(px * args.spp for _ in vals) / sum(dt for _, dt in vals) / MPX
    unit = "Mpx*spp/s"
    line = {
        "impl": "reference", "metric": "pathtracer Mpx*spp/s (config 1)", "value": value,
        "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(dt for _, dt in vals),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"config1 pathtracer {args.res}x{args.res} {args.spp}spp depth5 "
                               f"1015810 tris; each step renders a bounded sample of it: {rows} "
                               f"rows in 8 bands ({px} pixels) x {args.spp} spp, throughput "
                               "scaled per pixel-sample", "sample": f"{px} pixels per step"},
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port",
                         "sample": f"{px} of {args.res * args.res} pixels ({rows} rows in 8 bands) "
                                   f"x {args.spp} spp per step"},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    os.environ.setdefault("VISIONARAY_CUDA_DEVICE", str(local))
    pkg = importlib.import_module("anari-visionaray_gb300")
    vsr = pkg.vsr

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    scene = pkg.scenes.config1(res=args.res, spp=args.spp)
    scene["renderer"]["wavefront"] = args.wavefront
    scene["renderer"]["sampleChunks"] = args.sample_chunks
    if args.bvh_leaf_size is not None:
        scene["bvhLeafSize"] = args.bvh_leaf_size
    ntris = pkg.scenes.triangle_count(scene)
    dev = vsr.Device()
    h = pkg.scenes.build(dev, scene)
    frame = h["frame"]
    dev.set(h["renderer"], "sampleLimit", 1 << 30)
    dev.commit(h["renderer"])
    W, H = args.res, args.res
    px_samples = W * H * args.spp

    # first frame builds the BVH on the device (commit work, reported apart)
    dev.render(frame)
    dev.wait(frame)
    commit_s = dev.get_float(frame, "commitDuration")
    bvh_s = dev.get_float(h["world"], "bvh.buildDuration")

    # counting pass (untimed): rays, BVH node visits, triangle tests of one frame
    dev.set(frame, "collectStatistics", True)
    dev.commit(frame)
    dev.render(frame)
    dev.wait(frame)
    counts = dev.get_u64(frame, "statistics", 32) or [0] * 32
    dev.set(frame, "collectStatistics", False)
    dev.commit(frame)

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        dev.render(frame)
        dev.wait(frame)
    clocks = ClockSampler(local)
    clocks.start()
    durations = []
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        assert dev.render(frame) == 0
        dev.wait(frame)
        durations.append(dev.get_float(frame, "duration.render"))
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    err = dev.get_uint(frame, "errorFlags")
    iterations = dev.get_int(frame, "wavefrontIterations")

    # end to end through the public API with host buffers
    cam = h["camera"]
    c = scene["camera"]
    e2e_times = []
    d2h = W * H * (16 + 4 + 12 + 12)
    for i in range(args.e2e_steps + 1):
        pos = list(c["position"])
        pos[0] += 1e-3 * (i % 2)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t = time.perf_counter()
        dev.set(cam, "position", pos, vsr.FLOAT32_VEC3)
        dev.commit(cam)
        dev.render(frame)
        dev.wait(frame)
        for ch in ("channel.color", "channel.depth", "channel.normal", "channel.albedo"):
            dev.map_raw(frame, ch)
        if i > 0:
            e2e_times.append(time.perf_counter() - t)
    h2d = 3 * 4 + 4 * 4 * 0  # the camera position crosses to the device as kernel parameters
    # one frame at the scene's own camera, accumulation restarted: the same
    # random stream as the oracle's first frame (compared in the CPU leg)
    dev.set(cam, "position", list(c["position"]), vsr.FLOAT32_VEC3)
    dev.commit(cam)
    dev.render(frame)
    dev.wait(frame)
    first_frame = dev.map(frame, "channel.color") if world == 1 else None

    # the same samples as accumulated 1-spp frames (the reference's other way
    # to reach 64 spp): one frame per sample, L2 flushed before each
    accum = None
    if args.accum_frames > 0 and world == 1:
        dev.set(h["renderer"], "pixelSamples", 1)
        dev.set(h["renderer"], "sampleChunks", 1)
        dev.commit(h["renderer"])
        dev.render(frame)  # accumulation restarts after the commit
        dev.wait(frame)
        ad = []
        for _ in range(args.accum_frames):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            dev.render(frame)
            dev.wait(frame)
            ad.append(dev.get_float(frame, "duration.render"))
        accum = {"value": args.accum_frames * W * H / sum(ad) / MPX, "unit": "Mpx*spp/s",
                 "frames": args.accum_frames, "ms_per_frame": 1e3 * statistics.mean(ad),
                 "workload": f"config1 pathtracer {W}x{H}, {args.accum_frames} accumulated "
                             f"1-spp frames, L2 flushed before each"}
        dev.set(h["renderer"], "pixelSamples", args.spp)
        dev.set(h["renderer"], "sampleChunks", args.sample_chunks)
        dev.commit(h["renderer"])

    l2peak = measure_l2_read_peak(pkg) if args.raycast else None
    raycast = measure_raycast_config0(pkg, dev, flush, l2=l2peak) if args.raycast else None
    shaded = measure_raycast_config0(pkg, dev, flush, gradient=True) if args.raycast else None
    batch = measure_batch_config3(pkg, dev) if args.batch else None
    if not args.denoise:
        denoiser = None
    elif args.denoise_forward_only:
        denoiser = measure_denoiser_forward(pkg, dev)
    else:
        denoiser = measure_denoiser_config4(pkg, dev, train_scenes=args.denoise_train_scenes,
                                            eval_scenes=args.denoise_eval_scenes,
                                            steps=args.denoise_steps)
    volume = (measure_volume_config2(pkg, dev, flush, res=args.volume_res, spp=args.volume_spp,
                                     chunks=args.volume_sample_chunks, leaf_size=args.bvh_leaf_size)
              if args.volume else None)

    kernel_s = sum(durations) / len(durations)
    t_max = kernel_s
    if world > 1:
        tt = torch.tensor([kernel_s], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_max = float(tt.item())
    value = world * px_samples / t_max / MPX
    e2e_value = world * px_samples / statistics.mean(e2e_times) / MPX if e2e_times else None

    if rank != 0:
        dev.close()
        return
    rays, nodes, tris = counts[0], counts[1], counts[2]
    alg_bytes = nodes * 64 + tris * 48 + W * H * (16 + 16 + 4 + 12 + 12)
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / kernel_s / 1e9
    traffic = profiled_traffic()
    issue = issue_roofline(kernel_s, args.spp, args.res)
    line = {
        "metric": "pathtracer Mpx*spp/s (config 1)",
        "value": value, "unit": "Mpx*spp/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * kernel_s, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"config1 pathtracer {W}x{H} {args.spp}spp depth5 {ntris} tris",
                   "sample_chunks": args.sample_chunks,
                   "l2": "flushed (256 MiB write) between steps", "parallelism": f"replicas{world}"},
        "e2e": {"value": e2e_value, "unit": "Mpx*spp/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        # this library's kernels per timed frame: the megakernel and, with
        # sample chunks, kCombineChunks; in wavefront mode the init kernel and
        # a trace and a shade kernel per iteration (no accumulation reset
        # happens inside the timed loop)
        "gpu_launches": args.steps * ((1 + 2 * iterations) if args.wavefront and iterations
                                      else (2 if args.sample_chunks > 1 else 1)),
        # traversal and shading are issue- and latency-bound: thread
        # instructions per second against the SMs' lane-issue peak
        "roofline": dict(issue, traffic=traffic) if issue else
        {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
         "frac": achieved / peak, "traffic": traffic},
        "roofline_memory": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic,
                            "note": f"algorithmic bytes = BVH node fetches x64 B + triangle "
                                    f"fetches x48 B + frame bytes; peak {peak_kind}; most "
                                    "fetches hit L1/L2, so this is traversal memory work, not "
                                    "DRAM traffic"},
        "traversal": {"rays": rays, "node_visits": nodes, "tri_tests": tris,
                      "node_visit_histogram_log2": counts[8:24],
                      "grays_per_s": rays / kernel_s / 1e9,
                      **phase_split(counts)},
        "config1_accumulated_1spp": accum,
        "commit_s": commit_s, "bvh_build_s": bvh_s, "raycast_config0": raycast,
        "raycast_config0_gradient_shading": shaded,
        "volume_pathtracer_config2": volume, "batch_config3": batch,
        "denoiser_config4": denoiser,
        "wall_s_timed": wall, "clocks": clk, "error_flags": err,
        "wavefront_iterations": iterations,
    }
    if world == 1 and not args.no_cpu_baseline:
        v, dt, px, cores, rows, colour = cpu_baseline(scene, args.cpu_rows, keep=True)
        line["cpu_baseline"] = {"value": v, "unit": "Mpx*spp/s", "cores": cores, "kind": "port",
                                "sample": f"{px} of {W * H} pixels ({args.cpu_rows} rows in 8 bands) "
                                          f"x {args.spp} spp, {dt:.1f} s"}
        if first_frame is not None:
            # the CPU sample is the oracle's first frame of the same rows: the
            # GPU's first frame follows the same random streams
            g = np.concatenate([first_frame[a:b, :, :3] for a, b in rows])
            o = np.concatenate([colour[a:b, :, :3] for a, b in rows])
            d = np.abs(g.astype(np.float64) - o)
            line["cpu_baseline"]["parity"] = {
                "pixels": int(d.shape[0] * d.shape[1]),
                "within_1e-3": float((d.max(axis=-1) <= 1e-3).mean()),
                "rmse": float(np.sqrt(np.mean(d * d))), "mean_abs": float(d.mean()),
                "how": "GPU first frame vs the oracle's frame on the sampled rows, same "
                       "per-pixel random streams (accumulation restarted)"}
    print(json.dumps(line), flush=True)
    dev.close()


def run_batch_only():
    pkg = importlib.import_module("anari-visionaray_gb300")
    dev = pkg.vsr.Device()
    rec = measure_batch_config3(pkg, dev, profile_range=True)
    print(json.dumps({"batch_config3": rec}))
    dev.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.batch_only:
        run_batch_only()
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
