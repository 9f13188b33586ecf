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
  serving      request serving over 256 scenes (continuous batching, LRU
               device budget): saturation requests/s, p50/p99 latency under
               Poisson arrivals, an eviction run with a small budget.

``--impl reference`` times the CPU restatement alone on this workload (the
reference renderer itself is GL-only and cannot run here)."""
import argparse
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
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--envs", type=int, default=None)
    p.add_argument("--workload", default="config1", choices=["config1", "config2", "config3"],
                   help="config1 (the metric's workload) by default; config2/config3 for reference")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-replay", action="store_true")
    p.add_argument("--no-postprocess", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--serving-scenes", type=int, default=256)
    p.add_argument("--serving-requests", type=int, default=20000)
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
    "config1": WORKLOAD,
    "config2": ("config2 uneven batching: 4096 envs over 64 procedural scenes of 20k-2M triangles "
                "(log-uniform), per-env resolution 64/128/256 px (p 0.3/0.5/0.2), hfov U(60,110)"),
    "config3": ("config3 large scans: 256 envs over 8 scan-like rooms of 5.0M triangles each "
                "(noisy 1.31 cm tessellation, value-noise colour, 64 Voronoi ids), 256x256, "
                "random-walk cameras"),
}


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


def serving_leg(pkg, args):
    """Request serving over a catalog of procedural scenes (triangles
    log-uniform in 10k-1M, resolution 64/128/256 with p 0.3/0.5/0.2, 6-DoF
    poses): continuous batching into 96 + 64 + 16 render slots per step, one
    graph launch per step, slot rectangles copied back to pinned host memory
    overlapped with the next step.  A closed-loop run (every request pending
    at the start) gives the saturation rate; Poisson arrivals at 50 % and
    80 % of it give latency percentiles (arrival to images in host memory);
    a run with the device budget at a quarter of the catalog's bytes, Zipf(1)
    scene popularity and 500 requests/s exercises LRU eviction."""
    from habitat_sim_gb300 import server
    slots = {64: 96, 128: 64, 256: 16}
    cat = server.SceneCatalog(args.serving_scenes, seed=4, tri_range=(1e4, 1e6))
    t0 = time.perf_counter()
    assets = [cat.asset(s) for s in range(len(cat))]
    gen_s = time.perf_counter() - t0
    total_bytes = sum(a.device_bytes() for a in assets)
    tris = [a.triangles for a in assets]
    n = args.serving_requests
    out = {"workload": ("serving: %d procedural scenes (room shell + 20 boxes, %d-%d triangles, "
                        "mean %d, log-uniform), requests (scene, 6-DoF pose, 64/128/256 px "
                        "with p 0.3/0.5/0.2)" % (len(cat), min(tris), max(tris),
                                                  int(np.mean(tris)))),
           "slots": slots, "catalog_bytes": total_bytes, "catalog_generation_s": gen_s,
           "planes": "rgba8 + f32 linear depth + u32 semantic id per request",
           "latency": "arrival to all three images in host memory"}
    srv = server.RenderServer(pkg, cat, slots=slots, max_resident=len(cat),
                              budget_bytes=150 * 10**9)
    warm = server.random_requests(cat, max(len(cat), 2000), rate=0, seed=100)
    for s, q in enumerate(warm[:len(cat)]):
        q.scene = s                       # every scene resident before timing
    t0 = time.perf_counter()
    srv.serve(warm, realtime=False)
    out["warm_load_s"] = time.perf_counter() - t0

    def keep(st):
        return {k: st[k] for k in ("requests", "requests_per_s", "p50_ms", "p99_ms", "mean_ms",
                                   "mean_batch", "steps", "loads", "evictions", "elapsed_s")}
    sat = srv.serve(server.random_requests(cat, n, rate=0, seed=101), realtime=False)
    out["saturation"] = keep(sat)
    rate = sat["requests_per_s"]
    out["open_loop"] = []
    for k, frac in enumerate((0.5, 0.8)):
        st = srv.serve(server.random_requests(cat, n // 2, rate=frac * rate, seed=102 + k))
        out["open_loop"].append(dict(offered_per_s=frac * rate, **keep(st)))
    srv.close()
    budget = total_bytes // 4
    srv = server.RenderServer(pkg, cat, slots=slots, max_resident=len(cat), budget_bytes=budget)
    st = srv.serve(server.random_requests(cat, 2500, rate=500.0, seed=110, zipf=1.0))
    out["small_budget"] = dict(budget_bytes=budget, offered_per_s=500.0, popularity="zipf 1.0",
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
    m.close()
    return {"pixels": px,
            "redwood_noise": {"ms": noise_ms, "Gpx_per_s": px / noise_ms / 1e6,
                              "GB_per_s": 8 * px / noise_ms / 1e6,
                              "bytes_per_pixel": 8, "launches": 1},
            "hbao": {"ms": hbao_ms, "Gpx_per_s": px / hbao_ms / 1e6,
                     "GB_per_s": 24 * px / hbao_ms / 1e6, "bytes_per_pixel": 24, "launches": 3,
                     "note": "bytes: depth read by each of the 3 passes, 8-bit AO written and "
                             "read twice, colour read and written; the AO pass's 36 neighbour "
                             "depth reads per pixel are served by L1/L2"}}


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
        "config": {"workload": WORKLOADS[args.workload], "envs_per_step": per_step_envs,
                   "sample": f"first {per_step_envs} of {wl.envs} envs per step"},
        "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step_envs} envs per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the reference renderer is OpenGL-only (no GL, EGL or software rasteriser on "
                 "this machine); this arm times the C++ restatement of its draw path"),
    }
    print(json.dumps(line))
    return 0


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
    planes = pkg.Plane.Color | pkg.Plane.LinearDepth | pkg.Plane.Semantic
    r = procedural.build_renderer(pkg, wl, mode=pkg.DrawMode.Batched, planes=planes,
                                  double_buffer=True)
    r.setKernelTiming(True)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    steps = args.warmup + args.steps
    poses = [procedural.camera_poses(wl, i) for i in range(steps)]
    # Launch shape chosen by the autotuner (cached per GPU and workload), or
    # the library's default shape with --no-autotune.
    tune_report = {"cached": None, "trials": []}
    if not args.no_autotune:
        from habitat_sim_gb300 import autotune
        _, tune_report = autotune.tune(
            r, [procedural.camera_poses(wl, 1000 + i) for i in range(3)],
            int(wl.triangles_per_env().sum()),
            cache=os.path.join(ROOT, "habitat-sim_gb300", "_build", "autotune.json"))

    def batched_step(i, events=None):
        flush.zero_()
        r.updateCameras(*poses[i % steps])
        if events:
            events[0].record(stream)
        r.draw(stream=stream, mode=pkg.DrawMode.Batched, graph=True)
        if events:
            events[1].record(stream)

    for i in range(args.warmup):
        batched_step(i)
    torch.cuda.synchronize()

    # ---- timed batched steps
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    barrier_sync(world)
    step_ms, raster_ms, prepare_ms = [], [], []
    tri = None
    for k in range(args.steps):
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        batched_step(args.warmup + k, ev)
        st = r.lastDrawStats()          # synchronises the stream
        step_ms.append(ev[0].elapsed_time(ev[1]))
        raster_ms.append(st["raster_ms"])
        prepare_ms.append(st["prepare_ms"])
        tri = st["triangles"]
    barrier_sync(world)
    clocks = sampler.stop()
    total_ms = max_over_ranks(sum(step_ms), world)
    value = job_frames_per_s(wl.envs, args.steps, world, total_ms)

    # ---- plain per-scene path
    plain_ms = []
    for k in range(args.plain_steps + 1 if args.plain_steps else 0):
        r.updateCameras(*poses[k % steps])
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.draw(stream=stream, mode=pkg.DrawMode.PerScene)
        e1.record(stream)
        torch.cuda.synchronize()
        if k > 0:
            plain_ms.append(e0.elapsed_time(e1))
    plain_fps = wl.envs * len(plain_ms) / (sum(plain_ms) / 1e3) if plain_ms else None

    # ---- end to end through the C ABI with host buffers: every step takes
    # its poses from host arrays (uploaded in the step's camera block) and
    # reads its three planes back into pinned host memory; the readback of
    # step k runs on the renderer's copy stream from one set of planes while
    # step k + 1 draws into the other (double buffering).
    fbw, fbh = r.framebufferSize()

    def host_set():
        return (torch.empty((fbh, fbw, 4), dtype=torch.uint8, pin_memory=True).numpy(),
                torch.empty((fbh, fbw), dtype=torch.float32, pin_memory=True).numpy(),
                torch.empty((fbh, fbw), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32))
    hosts = [host_set(), host_set()]
    rect = ((0, 0), (fbw, fbh))
    readback = (pkg.Plane.Color, pkg.Plane.LinearDepth, pkg.Plane.Semantic)

    def e2e_step(k):
        r.updateCameras(*poses[k % steps])
        r.draw(stream=stream, mode=pkg.DrawMode.Batched, graph=True)
        for plane, buf in zip(readback, hosts[k % 2]):
            r.imageIntoAsync(plane, rect, buf)

    e2e_s = []
    n_e2e = args.e2e_steps
    if n_e2e:
        e2e_step(0)
        r.readbackWait()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(1, n_e2e + 1):
            e2e_step(k)
        r.readbackWait()
        e2e_s = [(time.perf_counter() - t0) / n_e2e] * n_e2e
    e2e_fps = wl.envs * len(e2e_s) / sum(e2e_s) if e2e_s else None
    host_color, host_lin, host_sem = hosts[n_e2e % 2]
    h2d = wl.envs * 96   # the camera block (P*V, view row, binding) per env
    d2h = host_color.nbytes + host_lin.nbytes + host_sem.nbytes

    # ---- parity of sampled envs against the oracle (last e2e step's poses)
    parity = None
    if rank == 0 and e2e_s:
        from oracle.model import OracleRenderer
        sample = [0, 1, 2, 3, wl.envs // 2 + 1, wl.envs - 1]
        cpu = procedural.build_oracle(OracleRenderer, wl, envs=sample)
        procedural.set_cameras(cpu, wl, poses[args.e2e_steps % steps], sample)
        cpu.draw(threads=os.cpu_count() or 1)
        mism, max_err, px = 0, 0.0, 0
        for slot, e in enumerate(sample):
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
                max_err = max(max_err, float(np.abs(g_lin[same].astype(np.float64) -
                                                    c_lin[same]).max()))
        parity = {"envs_checked": len(sample), "pixels": px, "mismatched_pixels": mism,
                  "max_linear_depth_err_m": max_err, "depth_tolerance_m": 1e-4}

    # ---- roofline of the raster kernel
    fb_bytes, geo_bytes = algorithmic_bytes(wl)
    launch_bytes = fb_bytes + geo_bytes
    raster_avg_ms = statistics.mean(raster_ms)
    achieved = launch_bytes / (raster_avg_ms / 1e3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    traffic = None
    tpath = os.path.join(ROOT, "profiles", f"raster_kernel_{args.workload}.txt")
    if os.path.exists(tpath):
        for line in open(tpath):
            if line.startswith("dram_bytes_per_launch:"):
                traffic = float(line.split(":")[1])

    post = None if args.no_postprocess else postprocess_leg(pkg, r, wl, stream)
    serving = None if args.no_serving else serving_leg(pkg, args)
    replay = None
    if not args.no_replay and wl.uniform:
        replay = replay_leg(pkg, procedural, wl, r.tuning())

    cpu_baseline = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        fps, n, dt = cpu_frames_per_s(procedural, wl, args.cpu_seconds, threads)
        cpu_baseline = {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port",
                        "sample": f"first {n} of {wl.envs} envs, one step, {dt:.2f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(step_ms),
            "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "envs": wl.envs,
                       "resolution": sorted({w for (w, _) in wl.viewports}),
                       "planes": "rgba8 + f32 linear depth + u32 semantic id",
                       "form": "batched: prepare + persistent raster per step, CUDA graph",
                       "l2": "flushed with a 256 MiB write before every step (outside timing)",
                       "triangles_per_step_after_draw_culling": tri,
                       "triangles_per_step_before_culling": int(wl.triangles_per_env().sum()),
                       "tuning": r.tuning(),
                       "autotune": None if args.no_autotune else {
                           "cached": tune_report["cached"],
                           "candidates": len(tune_report.get("trials", []))}},
            "plain": None if not plain_ms else {
                "value": plain_fps, "unit": "frames/s", "ms_per_step": statistics.mean(plain_ms),
                "p50_ms": float(np.percentile(plain_ms, 50)),
                "p99_ms": float(np.percentile(plain_ms, 99)),
                "form": "per-scene prepare + raster launches (2 per env), no graph"},
            "batched_over_plain": value / plain_fps if plain_fps else None,
            "e2e": None if not e2e_s else {
                "value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * statistics.mean(e2e_s),
                "timing": ("host clock over the steps: updateCameras + draw + 3 imageIntoAsync "
                           "readbacks per step, readback of step k overlapping the draw of "
                           "step k+1, then readbackWait")},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": peak_src, "kernel": "raster_kernel",
                         "bytes_per_launch": launch_bytes,
                         "bytes_breakdown": {"framebuffer": fb_bytes, "geometry_textures": geo_bytes},
                         "avg_launch_ms": raster_avg_ms,
                         "prepare_avg_ms": statistics.mean(prepare_ms)},
            "gpu_launches": 2 * args.steps,
            "clocks": clocks,
            "parity": parity,
            "cpu_baseline": cpu_baseline,
            "serving": serving,
            "replay": replay,
            "postprocess": post,
        }
        print(json.dumps(line))
    r.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
