#!/usr/bin/env python3
"""Throughput of the GB300 batch renderer on the textured-instancing workload.

One step renders every env of the workload once: 1024 envs over 4
procedural scenes (20k-triangle room + 200 textured instances each), 128 x 128
RGBA8 + FP32 linear depth + uint32 semantic id per env, fresh camera poses
every step (uploaded from host memory inside the step).

Printed (rank 0, one JSON line):
  value        frames/s of the batched form (one prepare + one persistent
               raster launch per step, replayed from a CUDA graph), geometry
               and textures resident in HBM, L2 flushed before every step
               (a 256 MiB write outside the timed events); each step timed
               with CUDA events on the launching stream;
  plain        the same workload through the plain per-scene path (two
               launches per env, no graph);
  e2e          the same metric through the C ABI with host buffers: poses
               from host arrays, framebuffer (colour, linear depth, ids) read
               back into pinned host memory by the imageInto calls;
  roofline     the raster kernel against measured HBM bandwidth, bytes = the
               framebuffer written plus the unique geometry and textures;
  cpu_baseline the CPU oracle (the renderer restated in C++) on a bounded
               sample of the same envs, all host threads;
  parity       sampled envs of the timed workload against the oracle;
  configs      the same measurements (batched, plain, e2e, roofline, parity
               sample, CPU oracle) for the other workloads: config0 (16 envs,
               one room), config2 (4096 envs, 64 scenes of 20k-2M triangles,
               mixed resolutions), config3 (256 envs of 5M-triangle scans,
               the 100-step camera walk);
  serving      request serving over 256 textured scenes (about 40 GB on the
               device; continuous batching, 150 GB budget with LRU
               eviction): saturation requests/s, p50/p99 latency under
               Poisson arrivals swept towards saturation, the plain
               one-request path, an eviction run with a small budget.

``--impl reference`` times the CPU restatement alone on this workload (the
reference renderer itself is GL-only and cannot run here)."""
import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "128² RGBD frames/s on 1 GB300, batched vs plain; p50/p99 ms at ≤1e-4 m depth err"
WORKLOAD = ("config1 textured instancing: 1024 envs over 4 procedural scenes, each a "
            "20,172-triangle room shell + 200 instances of 16 prototypes (500-5k tris, 512x512x16 "
            "RGBA8 noise texture array, bilinear), 128x128 pinhole hfov 90, near 0.01 far 10")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--plain-steps", type=int, default=3)
    p.add_argument("--e2e-steps", type=int, default=60)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--envs", type=int, default=None)
    p.add_argument("--workload", default="config1", choices=["config0", "config1", "config2", "config3"],
                   help="the main line's workload: config1 (the metric's) by default")
    p.add_argument("--configs", type=lambda t: [] if t in ("", "none") else t.split(","),
                   default=["config0", "config2", "config3"],
                   help="workloads measured as sub-blocks of the line (comma list, or none)")
    p.add_argument("--parity-envs", type=int, default=64)
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-replay", action="store_true")
    p.add_argument("--no-postprocess", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--serving-scenes", type=int, default=256)
    p.add_argument("--serving-requests", type=int, default=100000)
    p.add_argument("--serving-plain-requests", type=int, default=3000)
    p.add_argument("--serving-texture-side", type=int, default=2048)
    p.add_argument("--serving-fractions", type=lambda t: [float(x) for x in t.split(",")],
                   default=[0.1, 0.25, 0.5, 0.75, 0.9])
    p.add_argument("--serving-slots", default="64:96,128:160,256:64",
                   type=lambda t: {int(a): int(b) for a, b in (kv.split(":") for kv in t.split(","))},
                   help="render slots per square resolution, e.g. 64:96,128:64,256:16")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def barrier_sync(world):
    """All ranks at the same point with their GPU work finished."""
    import torch
    if world > 1:
        torch.distributed.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def max_over_ranks(value, world, device="cuda"):
    """The largest `value` over all ranks (every rank gets it).  Replicas
    render the same per-GPU work, so the job's time is the slowest rank's."""
    if world == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_frames_per_s(envs_per_rank, steps, world, total_ms_max):
    """Whole-job throughput: the frames of every rank over the slowest rank's time."""
    return envs_per_rank * steps * world / (total_ms_max / 1e3)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------- workload
WORKLOADS = {
    "config0": ("config0 plain small: 16 envs sharing one procedural room (8 x 8 x 3 m box of 64 x 64 "
                "quad grids, 49,152 triangles, + 20 boxes), per-vertex random RGB, per-object ids, "
                "128x128 pinhole hfov 90 at 1.25 m, uniform position and yaw"),
    "config1": WORKLOAD,
    "config2": ("config2 uneven batching: 4096 envs over 64 procedural scenes of 20k-2M triangles "
                "(log-uniform), per-env resolution 64/128/256 px (p 0.3/0.5/0.2), hfov U(60,110)"),
    "config3": ("config3 large scans: 256 envs over 8 scan-like rooms of 5.0M triangles each "
                "(noisy 1.31 cm tessellation, value-noise colour, 64 Voronoi ids), 256x256, "
                "random-walk cameras"),
}
PLANES = "rgba8 + f32 linear depth + u32 semantic id"


def workload_config(name, wl):
    """The ``config`` object of a JSON line: the same for both arms."""
    return {"workload": WORKLOADS[name], "envs": wl.envs,
            "resolution": sorted({w for (w, _) in wl.viewports}), "planes": PLANES}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def load_workload(name, envs=None):
    import __graft_entry__ as graft
    pkg = graft.build()
    from habitat_sim_gb300 import procedural
    kw = {} if envs is None else {"envs": envs}
    wl = getattr(procedural, name)(**kw)
    return pkg, procedural, wl


def algorithmic_bytes(wl):
    px = sum(w * h for (w, h) in wl.viewports)
    fb = px * 12   # RGBA8 + FP32 linear depth + uint32 id
    return fb, wl.geometry_bytes()


def cpu_frames_per_s(procedural, wl, seconds, threads):
    """The oracle on host cores over a growing sample of envs until the time budget."""
    from oracle.model import OracleRenderer
    n = 8
    best = None
    t_total = 0.0
    while True:
        envs = list(range(min(n, wl.envs)))
        cpu = procedural.build_oracle(OracleRenderer, wl, envs=envs)
        procedural.set_cameras(cpu, wl, procedural.camera_poses(wl, 0), envs)
        t0 = time.perf_counter()
        cpu.draw(threads=threads, window_depth=False)
        dt = time.perf_counter() - t0
        t_total += dt
        best = (len(envs), dt)
        if dt * 2.5 + t_total > seconds or len(envs) >= wl.envs:
            break
        n *= 2
    return best[0] / best[1], best[0], best[1]


def parity_envs(name, wl, count):
    """Envs checked against the oracle: spread over the scenes (config2: the
    envs of the largest scenes in every resolution class, and a spread of
    the rest)."""
    if name != "config2":
        step = max(1, wl.envs // count)
        return sorted({min(wl.envs - 1, i * step + i % 3) for i in range(count)})
    tri = wl.triangles_per_env()
    classes = sorted({w for (w, _) in wl.viewports})
    out = []
    for k, c in enumerate(classes):
        envs = [e for e in range(wl.envs) if wl.viewports[e][0] == c]
        envs.sort(key=lambda e: -int(tri[e]))
        take = count // len(classes) + (1 if k < count % len(classes) else 0)
        big = take // 2
        rest = envs[big:]
        out += envs[:big] + rest[::max(1, len(rest) // max(1, take - big))][:take - big]
    return sorted(set(out))


def check_parity(procedural, wl, r, host, envs, poses):
    """Sampled envs of one step (read back into `host`) against the oracle:
    pixels whose colour or id differ, largest linear-depth error where they agree."""
    from oracle.model import OracleRenderer
    host_color, host_lin, host_sem = host
    cpu = procedural.build_oracle(OracleRenderer, wl, envs=envs)
    procedural.set_cameras(cpu, wl, poses, envs)
    cpu.draw(threads=os.cpu_count() or 1)
    mism, max_err, px = 0, 0.0, 0
    for slot, e in enumerate(envs):
        off, pitch, w, h = r.sceneViewport(e)
        if wl.uniform:
            y0, x0 = off // pitch, off % pitch
            g_col = host_color[y0:y0 + h, x0:x0 + w]
            g_lin = host_lin[y0:y0 + h, x0:x0 + w]
            g_sem = host_sem[y0:y0 + h, x0:x0 + w]
        else:   # ragged: one row, scene after scene
            g_col = host_color[0, off:off + w * h].reshape(h, w, 4)
            g_lin = host_lin[0, off:off + w * h].reshape(h, w)
            g_sem = host_sem[0, off:off + w * h].reshape(h, w)
        c_col = cpu.scene_image(cpu.color, slot).view(np.uint8).reshape(h, w, 4)
        c_lin = cpu.scene_image(cpu.linear_depth, slot)
        c_sem = cpu.scene_image(cpu.semantic, slot)
        same = (g_col == c_col).all(-1) & (g_sem == c_sem)
        mism += int((~same).sum())
        px += same.size
        if same.any():
            max_err = max(max_err, float(np.abs(g_lin[same].astype(np.float64) - c_lin[same]).max()))
    return {"envs_checked": len(envs), "pixels": px, "mismatched_pixels": mism,
            "max_linear_depth_err_m": max_err, "depth_tolerance_m": 1e-4}


def measure(pkg, procedural, name, wl, steps, warmup, plain_steps, e2e_steps, parity_count, world=1,
            rank=0, local_rank=0, autotune=True, keep=False):
    """One workload: batched steps (CUDA graph, device-resident inputs, L2
    flushed before every step, CUDA events on the launching stream), the
    plain per-scene path, end to end through the C ABI with host buffers,
    the raster kernel's roofline, and a parity sample of the last e2e step.
    Returns (result dict, renderer if `keep` else None)."""
    import torch
    planes = pkg.Plane.Color | pkg.Plane.LinearDepth | pkg.Plane.Semantic
    r = procedural.build_renderer(pkg, wl, mode=pkg.DrawMode.Batched, planes=planes, double_buffer=True)
    r.setKernelTiming(True)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    n = warmup + max(steps, e2e_steps + 1)
    poses = [procedural.camera_poses(wl, i) for i in range(n)]
    tune_report = {"cached": None, "trials": []}
    if autotune:
        from habitat_sim_gb300 import autotune as at
        _, tune_report = at.tune(
            r, [procedural.camera_poses(wl, 1000 + i) for i in range(3)], int(wl.triangles_per_env().sum()),
            cache=os.path.join(ROOT, "habitat-sim_gb300", "_build", "autotune.json"))

    def batched_step(i, events=None):
        flush.zero_()
        r.updateCameras(*poses[i % n])
        if events:
            events[0].record(stream)
        r.draw(stream=stream, mode=pkg.DrawMode.Batched, graph=True)
        if events:
            events[1].record(stream)

    for i in range(warmup):
        batched_step(i)
    torch.cuda.synchronize()
    # The cyclic garbage collector stays off while steps are timed: a full
    # collection over the objects earlier workloads left would land inside
    # a timing window of a few tens of milliseconds.
    gc.collect()
    gc.disable()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    barrier_sync(world)
    step_ms, raster_ms, prepare_ms = [], [], []
    tri = None
    for k in range(steps):
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        batched_step(warmup + k, ev)
        st = r.lastDrawStats()          # synchronises the stream
        step_ms.append(ev[0].elapsed_time(ev[1]))
        raster_ms.append(st["raster_ms"])
        prepare_ms.append(st["prepare_ms"])
        tri = st["triangles"]
    barrier_sync(world)
    clocks = sampler.stop()
    total_ms = max_over_ranks(sum(step_ms), world)
    value = job_frames_per_s(wl.envs, steps, world, total_ms)

    # Plain per-scene path: one prepare + one raster launch per env, no graph.
    plain_ms = []
    for k in range(plain_steps + 1 if plain_steps else 0):
        r.updateCameras(*poses[k % n])
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.draw(stream=stream, mode=pkg.DrawMode.PerScene)
        e1.record(stream)
        torch.cuda.synchronize()
        if k > 0:
            plain_ms.append(e0.elapsed_time(e1))
    plain_fps = wl.envs * len(plain_ms) / (sum(plain_ms) / 1e3) if plain_ms else None
    t = r.tuning()
    plain_ctas = [-(-w // t["plain_region_width"]) * -(-h // t["plain_region_height"]) for (w, h) in wl.viewports]

    # End to end through the C ABI with host buffers: every step takes its
    # poses from host arrays (uploaded in the step's camera block) and reads
    # its three planes back into pinned host memory; the readback of step k
    # runs on the renderer's copy stream from one set of planes while step
    # k + 1 draws into the other (double buffering).
    fbw, fbh = r.framebufferSize()

    def host_set():
        return (torch.empty((fbh, fbw, 4), dtype=torch.uint8, pin_memory=True).numpy(),
                torch.empty((fbh, fbw), dtype=torch.float32, pin_memory=True).numpy(),
                torch.empty((fbh, fbw), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32))
    hosts = [host_set(), host_set()]
    rect = ((0, 0), (fbw, fbh))
    readback = (pkg.Plane.Color, pkg.Plane.LinearDepth, pkg.Plane.Semantic)

    def e2e_step(k):
        r.updateCameras(*poses[k % n])
        r.draw(stream=stream, mode=pkg.DrawMode.Batched, graph=True)
        for plane, buf in zip(readback, hosts[k % 2]):
            r.imageIntoAsync(plane, rect, buf)

    e2e_s, e2e_calls = None, []
    if e2e_steps:
        e2e_step(0)
        r.readbackWait()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        marks = [t0]
        for k in range(1, e2e_steps + 1):
            e2e_step(k)
            marks.append(time.perf_counter())
        r.readbackWait()
        marks.append(time.perf_counter())
        e2e_s = (marks[-1] - t0) / e2e_steps
        e2e_calls = [1e3 * (b - a) for a, b in zip(marks, marks[1:])]
    gc.enable()
    h2d = wl.envs * 96   # the camera block (P*V, view row, binding) per env
    d2h = sum(b.nbytes for b in hosts[0])
    parity = None
    if rank == 0 and e2e_steps and parity_count:
        parity = check_parity(procedural, wl, r, hosts[e2e_steps % 2], parity_envs(name, wl, parity_count),
                              poses[e2e_steps % n])

    fb_bytes, geo_bytes = algorithmic_bytes(wl)
    launch_bytes = fb_bytes + geo_bytes
    raster_avg = statistics.mean(raster_ms)
    achieved = launch_bytes / (raster_avg / 1e3) / 1e9
    peak, peak_src = 6800.0, "fallback"
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    traffic = None
    issue = None
    tpath = os.path.join(ROOT, "profiles", f"raster_kernel_{name}.txt")
    if os.path.exists(tpath):
        for line in open(tpath):
            if line.startswith("dram_bytes_per_launch:"):
                traffic = float(line.split(":")[1])
            elif line.startswith("smsp__issue_active.avg.pct_of_peak_sustained_active"):
                issue = float(line.split()[1]) / 100.0
    res = {
        "value": value, "unit": "frames/s", "steps": steps, "warmup": warmup,
        "ms_per_step": statistics.mean(step_ms), "p50_ms": float(np.percentile(step_ms, 50)),
        "p99_ms": float(np.percentile(step_ms, 99)),
        "plain": None if not plain_ms else {
            "value": plain_fps, "unit": "frames/s", "ms_per_step": statistics.mean(plain_ms),
            "p50_ms": float(np.percentile(plain_ms, 50)), "p99_ms": float(np.percentile(plain_ms, 99)),
            "ctas_per_env": {"min": min(plain_ctas), "max": max(plain_ctas),
                             "mean": float(np.mean(plain_ctas))},
            "form": "per-scene prepare + raster launches (2 per env, one env after another), no graph; "
                    "each env's raster launch is ctas_per_env CTAs of %d threads (%d x %d px regions)"
                    % (t["threads"], t["plain_region_width"], t["plain_region_height"])},
        "batched_over_plain": value / plain_fps if plain_fps else None,
        "e2e": None if e2e_s is None else {
            "value": wl.envs / e2e_s, "unit": "frames/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * e2e_s,
            "call_ms": [round(x, 3) for x in e2e_calls],
            "timing": ("host clock over the steps: updateCameras + draw + 3 imageIntoAsync readbacks per "
                       "step, readback of step k overlapping the draw of step k+1, then readbackWait; call_ms: "
                       "host time of each step's calls, the last entry readbackWait")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                     "issue_active_frac": issue,
                     "issue_note": ("the kernel is bound by instruction issue and latency, not HBM: "
                                    "share of cycles its schedulers issued (ncu capture in profiles/)")
                     if issue is not None else None,
                     "kernel": "raster_kernel", "bytes_per_launch": launch_bytes,
                     "bytes_breakdown": {"framebuffer": fb_bytes, "geometry_textures": geo_bytes},
                     "avg_launch_ms": raster_avg, "prepare_avg_ms": statistics.mean(prepare_ms),
                     "visible_draw_triangles_per_launch": tri,
                     "visible_draw_triangles_per_s": tri / (raster_avg / 1e3) if tri else None},
        "triangles_per_step_before_culling": int(wl.triangles_per_env().sum()),
        "tuning": t,
        "autotune": None if not autotune else {
            "cached": tune_report["cached"], "candidates": len(tune_report.get("trials", [])),
            "trials": [{k: tr.get(k) for k in ("threads", "region_width", "region_height", "small_area",
                                                "ctas_per_sm", "queue_fill_percent", "raster_ms", "error")
                        if tr.get(k) is not None} for tr in tune_report.get("trials", [])]},
        "clocks": clocks,
        "parity": parity,
        "gpu_launches": 2 * steps,
    }
    del flush
    if keep:
        return res, r
    r.close()
    return res, None


def serving_leg(pkg, args):
    """Request serving on the serving workload: a catalog of 256 procedural
    scenes (a 12 x 3 x 12 m room shell + 20 boxes, triangles log-uniform in
    10k-1M, one 2048 x 2048 RGBA8 uniform-noise texture layer per 24k
    triangles sampled bilinear, one mesh view and material per object: about
    40 GB of geometry and textures on the device), requests (scene uniform,
    6-DoF pose, 64/128/256 px with p 0.3/0.5/0.2), a 150 GB device budget with
    LRU eviction.  Continuous batching into 96 + 160 + 64 render slots per
    step (320 requests of the resolution mix), one graph launch per step,
    slot rectangles copied back to pinned host memory overlapped with the
    next step.  Runs: every scene loaded
    (timed); the launch shape chosen by closed-loop throughput (the
    autotuner's search space); a closed-loop run of all requests (saturation); Poisson arrivals
    at fractions of saturation (the sweep; latency from arrival to the three
    images in pinned host memory); the plain path (one request per draw) on a
    closed-loop sample; a run with the budget at a quarter of the catalog's
    bytes, Zipf(1) popularity and 200 requests/s, where eviction works
    (after an untimed run of the same popularity: steady state)."""
    from habitat_sim_gb300 import server
    slots = dict(args.serving_slots)
    n = args.serving_requests
    t0 = time.perf_counter()
    cat = server.SceneCatalog(args.serving_scenes, seed=4, tri_range=(1e4, 1e6),
                              texture_side=args.serving_texture_side)
    assets = [cat.asset(s) for s in range(len(cat))]
    gen_s = time.perf_counter() - t0
    total_bytes = sum(a.device_bytes() for a in assets)
    tex_bytes = sum(a.texture.size for a in assets)
    tris = [a.triangles for a in assets]
    out = {"workload": ("serving: %d procedural scenes (room shell + 20 boxes, %d-%d triangles, mean %d, "
                        "log-uniform; %d x %d RGBA8 noise texture layers, one per 24k triangles, bilinear), "
                        "requests (scene uniform, 6-DoF pose, 64/128/256 px with p 0.3/0.5/0.2)"
                        % (len(cat), min(tris), max(tris), int(np.mean(tris)), args.serving_texture_side,
                           args.serving_texture_side)),
           "slots": slots, "catalog_bytes": total_bytes, "catalog_texture_bytes": tex_bytes,
           "catalog_geometry_bytes": total_bytes - tex_bytes, "catalog_generation_s": gen_s,
           "budget_bytes": 150 * 10**9, "requests_per_run": n,
           "planes": "rgba8 + f32 linear depth + u32 semantic id per request",
           "latency": "arrival to all three images in pinned host memory"}
    srv = server.RenderServer(pkg, cat, slots=slots, max_resident=len(cat), budget_bytes=150 * 10**9,
                              max_loads_per_step=len(cat))
    warm = server.random_requests(cat, len(cat), rate=0, seed=100)
    for s, q in enumerate(warm):
        q.scene = s                       # every scene resident before timing
    t0 = time.perf_counter()
    srv.serve(warm, realtime=False, keep_images=False)
    out["warm_load_s"] = time.perf_counter() - t0
    out["resident_bytes"] = int(srv.residency.bytes)
    out["device_bytes_held"] = int(srv.r.deviceMemory()[0])
    if not args.no_autotune:
        tuning, trials = srv.tune(lambda: server.random_requests(cat, 3000, rate=0, seed=130))
        out["tuning"] = tuning
        out["autotune"] = {"objective": "closed-loop requests/s serving 3000 requests",
                           "trials": trials}

    def keep(st, closed=False):
        # A closed-loop run has every request pending at the start: its
        # latencies are queueing time, so only its throughput is reported.
        keys = ("requests", "requests_per_s", "mean_batch", "steps", "loads", "evictions", "elapsed_s")
        return {k: st[k] for k in keys + (() if closed else ("p50_ms", "p99_ms", "mean_ms"))}
    sat = srv.serve(server.random_requests(cat, n, rate=0, seed=101), realtime=False, keep_images=False)
    out["saturation"] = dict(keep(sat, closed=True), form="closed loop: all requests pending at the start")
    rate = sat["requests_per_s"]
    out["sweep"] = []
    for k, frac in enumerate(args.serving_fractions):
        st = srv.serve(server.random_requests(cat, n, rate=frac * rate, seed=102 + k), keep_images=False)
        out["sweep"].append(dict(fraction=frac, offered_per_s=frac * rate, **keep(st)))
    plain = srv.serve(server.random_requests(cat, args.serving_plain_requests, rate=0, seed=120),
                      realtime=False, keep_images=False, max_batch=1)
    out["plain"] = dict(keep(plain, closed=True), form="one request per step (one draw per request), closed loop")
    out["saturation_over_plain"] = rate / plain["requests_per_s"]
    srv.close()
    budget = total_bytes // 4
    srv = server.RenderServer(pkg, cat, slots=slots, max_resident=len(cat), budget_bytes=budget)
    if "tuning" in out:
        srv.r.setTuning(**out["tuning"])
    # Steady state: an untimed run of the same popularity fills the budget
    # first, so that the timed run measures eviction, not the cold start.
    srv.serve(server.random_requests(cat, 1000, rate=200.0, seed=111, zipf=1.0), keep_images=False)
    st = srv.serve(server.random_requests(cat, 1000, rate=200.0, seed=110, zipf=1.0), keep_images=False)
    out["small_budget"] = dict(budget_bytes=budget, offered_per_s=200.0, popularity="zipf 1.0",
                               warmed="an untimed run of 1000 requests of the same popularity first",
                               **keep(st))
    srv.close()
    return out


def postprocess_leg(pkg, r, wl, stream, reps=10):
    """Device time of the depth-noise model and of ambient occlusion over
    every env of the last draw (CUDA events on the launching stream)."""
    import torch
    from habitat_sim_gb300 import noise
    px = sum(w * h for (w, h) in wl.viewports)
    m = noise.RedwoodNoiseModelGPUImpl(noise.load_model(), torch.cuda.current_device(), 1.0, seed=1)
    dst = torch.empty_like(r.linearDepthTensor())

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    noise_ms = timed(lambda: m.apply_to_renderer(r, dst, stream.cuda_stream))
    hbao_ms = timed(lambda: r.drawHbao(stream=stream))
    variants = {}
    for name, cfg in (("cache_aware", pkg.HbaoConfiguration().setAlgorithm(pkg.HbaoType.CacheAware)),
                      ("special_blur", pkg.HbaoConfiguration().setUseSpecialBlur(True)),
                      ("cache_aware_special_blur",
                       pkg.HbaoConfiguration().setAlgorithm(pkg.HbaoType.CacheAware).setUseSpecialBlur(True))):
        ms = timed(lambda: r.drawHbao(cfg, stream=stream))
        variants[name] = {"ms": ms, "Gpx_per_s": px / ms / 1e6}
    m.close()
    return {"pixels": px,
            "redwood_noise": {"ms": noise_ms, "Gpx_per_s": px / noise_ms / 1e6,
                              "GB_per_s": 8 * px / noise_ms / 1e6,
                              "bytes_per_pixel": 8, "launches": 1},
            "hbao": {"ms": hbao_ms, "Gpx_per_s": px / hbao_ms / 1e6,
                     "GB_per_s": 24 * px / hbao_ms / 1e6, "bytes_per_pixel": 24, "launches": 3,
                     "note": "bytes: depth read by each of the 3 passes, 8-bit AO written and "
                             "read twice, colour read and written; the AO pass's 36 neighbour "
                             "depth reads per pixel are served by L1/L2",
                     "variants": variants}}


def replay_leg(pkg, procedural, wl, tuning, steps=5, warmup=2):
    """The replay path (BatchReplayRenderer through keyframes): every env is
    created from a scene keyframe, then each step applies one serialized
    camera keyframe per env (C++ parse + apply + camera from the user
    transform) and renders every env's colour and metres depth into pinned
    host images."""
    import torch
    cfg = pkg.ReplayRendererConfiguration()
    cfg.num_environments = wl.envs
    w, h = wl.viewports[0]
    cfg.sensor_specifications = [pkg.CameraSensorSpec(resolution=(h, w), hfov=float(wl.hfov[0]),
                                                      near=procedural.NEAR, far=procedural.FAR)]
    cfg.quiet = True
    rr = pkg.ReplayRenderer.create_batch_replay_renderer(cfg)
    rr.renderer.setTuning(**tuning)      # the batched leg's (autotuned) launch shape
    procedural.add_resources(rr.renderer, wl)
    t0 = time.perf_counter()
    scene_kf = [procedural.scene_keyframe(pkg, wl, s).to_string() for s in range(len(wl.instances))]
    for e in range(wl.envs):
        rr.set_environment_keyframe(e, scene_kf[wl.scene_of_env[e]])
    load_s = time.perf_counter() - t0
    n = warmup + steps
    cams = []
    for i in range(n):
        _, views = procedural.camera_poses(wl, 2000 + i)
        cams.append([procedural.camera_keyframe(pkg, views[e]).to_string() for e in range(wl.envs)])
    big_c = torch.empty((wl.envs, h, w, 4), dtype=torch.uint8, pin_memory=True).numpy()
    big_d = torch.empty((wl.envs, h, w), dtype=torch.float32, pin_memory=True).numpy()

    def step(i, batch):
        t = time.perf_counter()
        if batch:
            rr.set_environment_keyframes_batch(cams[i], sensor_prefix="sensor_")
        else:
            for e in range(wl.envs):
                rr.set_environment_keyframe(e, cams[i][e])
                rr.set_sensor_transforms_from_keyframe(e, "sensor_")
        t1 = time.perf_counter()
        rr.render(big_c, big_d)
        return t1 - t, time.perf_counter() - t1

    out = {}
    for batch in (False, True):
        apply_s, render_s = [], []
        for i in range(warmup):
            step(i, batch)
        for i in range(warmup, n):
            a, b = step(i, batch)
            apply_s.append(a)
            render_s.append(b)
        total = sum(apply_s) + sum(render_s)
        out[batch] = {"value": wl.envs * steps / total, "ms_per_step": 1e3 * total / steps,
                      "keyframe_apply_ms": 1e3 * statistics.mean(apply_s),
                      "render_ms": 1e3 * statistics.mean(render_s)}
    rr.close()
    res = dict(out[False])
    res.update({"unit": "frames/s", "envs": wl.envs, "steps": steps, "scene_load_s": load_s,
                "d2h_bytes_per_step": int(big_c.nbytes + big_d.nbytes),
                "timing": "host clock: per env set_environment_keyframe + "
                          "set_sensor_transforms_from_keyframe, then render() into pinned host images"})
    res["batched_keyframes"] = dict(out[True], timing="host clock: one set_environment_keyframes_batch "
                                    "call (parse + apply + sensor transforms for every env), then render()")
    return res


def run_reference_impl(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__ as graft
    graft.load_package()
    from oracle import build as oracle_build
    oracle_build.build()
    from habitat_sim_gb300 import procedural
    from oracle.model import OracleRenderer
    wl = getattr(procedural, args.workload)(**({} if args.envs is None else {"envs": args.envs}))
    threads = os.cpu_count() or 1
    # Size one step so that warmup + steps end within a few minutes.
    fps, n, dt = cpu_frames_per_s(procedural, wl, min(args.cpu_seconds, 8.0), threads)
    per_step_envs = max(1, min(wl.envs, int(fps * 4.0)))
    envs = list(range(per_step_envs))
    cpu = procedural.build_oracle(OracleRenderer, wl, envs=envs)
    times = []
    for i in range(args.warmup + args.steps):
        procedural.set_cameras(cpu, wl, procedural.camera_poses(wl, i), envs)
        t0 = time.perf_counter()
        cpu.draw(threads=threads, window_depth=False)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = per_step_envs * len(times) / sum(times)
    ms = [t * 1e3 for t in times]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(ms), "p50_ms": float(np.percentile(ms, 50)),
        "p99_ms": float(np.percentile(ms, 99)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.workload, wl),
        "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "cpu_model": cpu_model(),
                         "kind": "port",
                         "sample": f"first {per_step_envs} of {wl.envs} envs per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the reference renderer is OpenGL-only (no GL, EGL or software rasteriser on "
                 "this machine); this arm times the C++ restatement of its draw path"),
    }
    print(json.dumps(line))
    return 0


# Per-config sub-blocks of the default run: (steps, warmup, plain steps, e2e
# steps, envs checked against the oracle).  config3's 100 steps are its
# stated 100-step camera walk.  The end-to-end windows run for a few hundred
# milliseconds, so that the final readback (which nothing overlaps) and a
# rare host stall of a few milliseconds do not dominate them.
SUB_CONFIGS = {"config0": (20, 3, 3, 40, 16), "config2": (10, 3, 1, 60, 16), "config3": (100, 3, 1, 60, 8)}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference_impl(args)
    rank, local_rank, world = dist_env()
    import torch
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    pkg, procedural, wl = load_workload(args.workload, args.envs)
    main_res, r = measure(pkg, procedural, args.workload, wl, args.steps, args.warmup, args.plain_steps,
                          args.e2e_steps, args.parity_envs, world, rank, local_rank,
                          autotune=not args.no_autotune, keep=True)
    stream = torch.cuda.current_stream()
    post = None if args.no_postprocess else postprocess_leg(pkg, r, wl, stream)
    tuning = r.tuning()
    r.close()
    replay = None
    if not args.no_replay and wl.uniform:
        replay = replay_leg(pkg, procedural, wl, tuning)
    configs = {}
    if world == 1:
        for name in args.configs:
            if name == args.workload:
                continue
            steps, warmup, plain, e2e, par = SUB_CONFIGS[name]
            sub_wl = getattr(procedural, name)()
            res, _ = measure(pkg, procedural, name, sub_wl, steps, warmup, plain, e2e, par,
                             autotune=not args.no_autotune)
            res["config"] = workload_config(name, sub_wl)
            if not args.no_cpu_baseline:
                threads = os.cpu_count() or 1
                fps, n_cpu, dt = cpu_frames_per_s(procedural, sub_wl, 4.0, threads)
                res["cpu_baseline"] = {"value": fps, "unit": "frames/s", "cores": threads,
                                       "cpu_model": cpu_model(), "kind": "port",
                                       "sample": f"first {n_cpu} of {sub_wl.envs} envs, one step, {dt:.2f} s"}
            configs[name] = res
            del sub_wl
    serving = None if args.no_serving else serving_leg(pkg, args)

    cpu_baseline = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        fps, n, dt = cpu_frames_per_s(procedural, wl, args.cpu_seconds, threads)
        cpu_baseline = {"value": fps, "unit": "frames/s", "cores": threads, "cpu_model": cpu_model(),
                        "kind": "port", "sample": f"first {n} of {wl.envs} envs, one step, {dt:.2f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": main_res["value"], "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": main_res["ms_per_step"],
            "p50_ms": main_res["p50_ms"], "p99_ms": main_res["p99_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(args.workload, wl),
            "details": {"form": "batched: prepare + persistent raster per step, CUDA graph",
                        "l2": "flushed with a 256 MiB write before every step (outside timing)",
                        "triangles_per_step_before_culling": main_res["triangles_per_step_before_culling"],
                        "tuning": main_res["tuning"], "autotune": main_res["autotune"]},
            "plain": main_res["plain"],
            "batched_over_plain": main_res["batched_over_plain"],
            "e2e": main_res["e2e"],
            "roofline": main_res["roofline"],
            "gpu_launches": main_res["gpu_launches"],
            "clocks": main_res["clocks"],
            "parity": main_res["parity"],
            "cpu_baseline": cpu_baseline,
            "configs": configs,
            "serving": serving,
            "replay": replay,
            "postprocess": post,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
