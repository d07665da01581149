"""Benchmark of the GB300 vertex stage (visible triangles per second).

Default workload: the batched form -- 4096 models with log-uniform vertex
counts in [24, 65536] (35.1M vertices, 69.7M triangles), 32 point lights +
ambient with a random LightGroup per model, 1920x1080 camera, animated
transforms -- rendered as one persistent launch per phase (the launch shape and
tile size picked by the autotuner) and replayed from a captured CUDA graph. A
step is one frame over all 4096 models.

  value  visible triangles/s with the scene resident in HBM (graph replay)
  e2e    the same metric through the public C ABI with host buffers: per step
         the host pushes every model transform (t3d_scene_set_models), renders
         (t3d_render, batched) and reads the per-pair visible counts back
         (t3d_frame_readback + t3d_frame_collect, pipelined one frame deep)
  plain  one launch per render pair (the reference's render + flush loop)

python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                [--workload batched|terrain|cubes|sphere|serving]
Under torchrun (N > 1) every rank renders its own replica (replicas only: the
stage has no cross-GPU exchange); rank 0 prints the JSON line.
"""
import argparse
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

METRIC = "visible_tris_per_s"
UNIT = "tris/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_model():
    """The host CPU's model name (lscpu), stated beside the CPU arms' core counts."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def make_scene(workload, models=4096):
    from tetra3d_gb300 import scenes
    if workload == "batched":
        return scenes.batched_scene(4, n=models)
    if workload == "terrain":
        return scenes.terrain_scene(3)
    if workload == "cubes":
        return scenes.cubes_scene(2)
    if workload == "sphere":
        return scenes.uv_sphere_scene(1)
    raise ValueError(workload)


def workload_config(workload, sd):
    c = sd.camera
    base = {"workload": {"batched": f"batched_{sd.nmodels}_models", "terrain": "terrain_grid_1024x1024",
                         "cubes": "cubes_1000", "sphere": "uv_sphere_32x16"}[workload],
            "models": int(sd.nmodels), "vertices": int(sd.total_verts()), "triangles": int(sd.total_tris()),
            "camera": f"{c.width}x{c.height} fov{c.fov_y:g}", "lights": int(sd.nlights),
            "l2": "inputs larger than L2 (129 MB), no flush" if sd.total_verts() * 48 > 256e6 else
                  "small scene: L2-resident across steps (no flush)"}
    return base


def time_cpu(sd, cam, threads, animated, min_seconds=10.0, max_reps=50, first_frame=1):
    """The oracle (the reference's path restated on the CPU) on whole frames of the workload:
    frame k applies every model's animation step k times, as the k-th graph replay does. The
    output arrays are allocated and touched once before the timed frames (the reference's
    render loop reuses its scratch and vertex lists). Repeats until min_seconds have passed.
    Returns (visible tris/s, frames, seconds)."""
    from oracle import pyoracle
    r = pyoracle.Renderer(sd, cam)
    r.render(animate_frames=first_frame if animated else 0, threads=threads)
    reps, vis, t0 = 0, 0, time.perf_counter()
    while True:
        vis += r.render(animate_frames=(first_frame + reps) if animated else 0, threads=threads)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= max_reps:
            break
    return vis / el, reps, el


# ----------------------------------------------------------------- ours ----
def run_ours(args, rank, world, local_rank):
    import ctypes as C

    import torch
    import __graft_entry__
    from tetra3d_gb300 import abi, replicas, scenes
    from tetra3d_gb300.runtime import Context

    __graft_entry__.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    sd = make_scene(args.workload, args.models)
    if args.textured:  # raster textures on every material (the vertex stage does not change)
        scenes.texture_materials(sd, 7)
    ctx = Context(local_rank)
    if args.textured:
        ctx.set_textures(scenes.raster_textures())
    sid = ctx.upload(sd)
    cam = sd.camera
    animate = args.workload == "batched"
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
            torch.cuda.synchronize()

    # the autotuner picks the launch shape (one launch per phase or one cooperative launch) and
    # the tile size on this scene before the timed region
    tuned = None
    if not args.no_tune:
        from tetra3d_gb300 import autotune
        a0 = time.perf_counter()
        best, res = autotune.tune(ctx, sid, cam, frames=5, animate=False, chunks=())
        tuned = {"tile_tris": best[0], "block_threads": best[1], "split_phases": best[2],
                 "sweep_ms": {f"tile{k[0]}_block{k[1]}_split{k[2]}": round(v, 4) for k, v in res.items()},
                 "seconds": round(time.perf_counter() - a0, 1)}
        ctx.set_models(sid, sd)  # restore the initial transforms after the sweep
    split_used = tuned["split_phases"] if tuned else 1
    tile_used = tuned["tile_tris"] if tuned else 2048
    # ---- device-resident value: captured CUDA graph of the batched frame ----
    ctx.graph_capture(sid, cam, animate=animate)
    ctx.graph_replay(args.warmup, stream=sh)
    torch.cuda.synchronize()
    v0, b0 = ctx.counters()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        ev0.record(stream)
        ctx.graph_replay(args.steps, stream=sh)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    v1, b1 = ctx.counters()
    vis = v1 - v0
    alg_bytes = (b1 - b0) + 108 * vis
    ms, vis, alg_bytes = replicas.combine(ms, vis, alg_bytes, dist, device="cuda")
    value = vis / (ms / 1e3)
    ms_per_step = ms / args.steps
    st_last = ctx.sync()

    # ---- plain path: one launch per render pair ----
    plain = None
    if rank == 0 and not args.no_plain:
        pf = max(1, min(3, args.steps))
        ctx.render(sid, cam, mode=abi.MODE_PLAIN, animate=False, stream=sh)
        ctx.sync()
        pv0, _ = ctx.counters()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(pf):
            ctx.render(sid, cam, mode=abi.MODE_PLAIN, animate=False, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        pst = ctx.sync()
        pv1, _ = ctx.counters()
        pms = e0.elapsed_time(e1) / pf
        plain = {"tris_per_s": (pv1 - pv0) / (pms * pf / 1e3), "ms_per_frame": pms,
                 "launches_per_frame": int(pst.launches), "frames": pf}

    # ---- e2e through the public API with host buffers ----
    e2e = None
    if rank == 0:
        n = sd.nmodels
        rot = sd.mv["rotation"].reshape(n, 4, 4).copy()
        step = sd.mv["rotate_step"].reshape(n, 4, 4).copy()
        ek = max(3, min(args.steps, 30))
        # warm
        ctx.set_models(sid, sd)
        ctx.render(sid, cam, mode=abi.MODE_BATCHED, stream=sh)
        ctx.sync()
        ev, eb = 0, 0
        h2d = d2h = 0
        tm = {"game_loop_rotate": 0.0, "set_models": 0.0, "render_call": 0.0, "sync": 0.0}

        def push():
            a1 = time.perf_counter()
            ctx.set_models(sid, sd)  # queued on the device behind the frame in flight
            tm["set_models"] += time.perf_counter() - a1

        def render():
            a2 = time.perf_counter()
            ctx.render(sid, cam, mode=abi.MODE_BATCHED, stream=sh)
            tm["render_call"] += time.perf_counter() - a2

        # A pipelined game loop: frame i's read-back of its per-pair counts is queued right
        # behind it; while the GPU renders frame i the host advances the transforms of frame
        # i + 1 (Node.Rotate) and pushes them (the copy is queued behind frame i and its
        # read-back), queues frame i + 1, and only then collects frame i's counts, so the GPU
        # goes from one frame to the next without waiting for the host.
        t0 = time.perf_counter()
        push()
        render()
        for i in range(ek):
            ctx.readback()
            a0 = time.perf_counter()
            nxt = scenes.mult(step, rot) if (animate and i + 1 < ek) else rot
            tm["game_loop_rotate"] += time.perf_counter() - a0
            if i + 1 < ek:
                rot = nxt
                sd.mv["rotation"] = rot.reshape(n, 16)
                push()
                render()
            a1 = time.perf_counter()
            st = ctx.collect()
            tm["sync"] += time.perf_counter() - a1
            ev += st.visible_tris
            h2d += n * C.sizeof(abi.ModelDesc) + st.h2d_bytes
            d2h += st.d2h_bytes
        ctx.sync()
        el = time.perf_counter() - t0
        e2e = {"value": ev / el, "unit": UNIT, "h2d_bytes_per_step": int(h2d // ek),
               "d2h_bytes_per_step": int(d2h // ek), "ms_per_step": el / ek * 1e3, "steps": ek,
               "host_ms_per_step": {k: round(v / ek * 1e3, 3) for k, v in tm.items()}}

    # ---- rasterising the last frame's stream (colour + depth passes of flush) ----
    raster = None
    if rank == 0 and not args.no_raster:
        ctx.render(sid, cam, mode=abi.MODE_BATCHED, stream=sh)
        rst = ctx.sync()
        col, dep = ctx.raster(stream=sh)
        reps = 3
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        r0 = time.perf_counter()
        e0.record(stream)
        for _ in range(reps):
            ctx.raster(download=False, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        rms = (time.perf_counter() - r0) / reps * 1e3
        rdev = e0.elapsed_time(e1) / reps
        # algorithmic bytes: every visible triangle's three corners read once (xyuv, rgba, depth:
        # 108 B), the colour and depth images written once (8 B per pixel)
        rbytes = 108 * int(rst.visible_tris) + 8 * cam.width * cam.height
        rpeak, rpeak_kind = peaks()
        # the raster oracle (one host thread) on the same stream, downloaded
        from oracle import pyoracle
        fr = ctx.download(rst)
        c0 = time.perf_counter()
        pyoracle.raster(fr, sd, cam, textures=scenes.raster_textures() if args.textured else None)
        rcpu = {"value": int(rst.visible_tris) / (time.perf_counter() - c0), "unit": "tris/s", "cores": 1, "kind": "port",
                "sample": "the whole frame's stream, 1 rasterisation"}
        del fr
        raster = {"textured": bool(args.textured), "cpu_baseline": rcpu, "ms_per_frame": rms, "device_ms_per_frame": rdev, "image": f"{cam.width}x{cam.height}",
                  "visible_tris": int(rst.visible_tris), "tris_per_s": int(rst.visible_tris) / (rms / 1e3),
                  "covered_pixels": int((col[..., 3] > 0).sum()),
                  "roofline": {"bound": "hbm", "achieved": rbytes / (rdev / 1e3) / 1e9, "peak": rpeak, "unit": "GB/s",
                               "frac": rbytes / (rdev / 1e3) / 1e9 / rpeak, "algorithmic_bytes": rbytes,
                               "peak_source": f"{rpeak_kind} hbm_gbs"},
                  "note": "t3d_frame_raster (fragments, counting sort by pixel, per-pixel draw-order passes): ms_per_frame is "
                          "wall time incl. its host syncs, device_ms_per_frame CUDA events on its stream"}

    # ---- the frame with one vertex-stage feature on for every model ----
    features = None
    if rank == 0 and not args.no_features and args.workload == "batched" and args.models == 4096:
        ctx.release(sid)
        sid = None
        features = feature_frames(ctx, stream, sh, ms_per_step)

    # ---- serving sweep (continuous batching over 64 resident scenes) ----
    serve = None
    if rank == 0 and not args.no_serving and args.workload == "batched":
        if sid is not None:
            ctx.release(sid)
            sid = None
        serve = serving_sweep(ctx, [int(r) for r in args.rates.split(",")], args.serve_seconds,
                              args.serve_max_requests)

    # ---- CPU baseline (the oracle port on all host threads, whole frames of the same workload) ----
    cpu = cpu1 = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, reps, el = time_cpu(sd, cam, threads, animate, min_seconds=args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "cpu_model": cpu_model(), "kind": "port",
               "sample": f"{reps} whole frames ({sd.nmodels} models{', animated' if animate else ''}) in {el:.1f} s"}
        # the reference's Render is one goroutine: the same port on one host thread, over every
        # 8th model of the frame (render pairs are independent, so the sample's rate is the frame's)
        from oracle import pyoracle
        sub = scenes.subset(sd, np.arange(0, sd.nmodels, 8)) if sd.nmodels >= 64 else sd
        r1 = pyoracle.Renderer(sub, cam)
        r1.render(animate_frames=1 if animate else 0, threads=1)  # the output arrays touched once
        c0 = time.perf_counter()
        vis1 = r1.render(animate_frames=1 if animate else 0, threads=1)
        el1 = time.perf_counter() - c0
        del r1
        cpu1 = {"value": vis1 / el1, "unit": UNIT, "cores": 1, "cpu_model": cpu_model(), "kind": "port",
                "sample": f"one frame of every 8th model ({sub.nmodels} models) on one host thread, {el1:.1f} s"}

    if rank == 0:
        peak, peak_kind = peaks()
        achieved = alg_bytes / (ms / 1e3) / 1e9 / max(1, world)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": dict(workload_config(args.workload, sd),
                           form=("batched: one persistent launch per phase" if split_used else
                                 "batched: one cooperative persistent launch") + ", CUDA graph replay",
                           tile_tris=tile_used, animated=animate,
                           parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_step": alg_bytes / args.steps / max(1, world),
                         "traffic_note": "DRAM bytes per launch are not measurable inside this run (ncu only); "
                                         "the capture of this kernel is summarised in profiles/"},
            "cpu_baseline": cpu,
            "cpu_baseline_single_thread": cpu1,
            "e2e": e2e,
            "clocks": clk.summary(),
            "gpu_launches": int(args.steps) * int(st_last.launches),
            "launches_per_frame": int(st_last.launches),
            "visible_tris_per_step": vis / args.steps / max(1, world),
            "culled_models_last_frame": int(st_last.culled_models),
            "phase_us_last_frame": {k: round(float(v), 1) for k, v in
                                    zip(("prep", "vertex", "triangles", "hist", "scan", "rank_emit"), st_last.phase_us)},
            "phase_busy_us_last_frame": {k: round(float(v), 1) for k, v in
                                         zip(("prep", "vertex", "triangles", "hist", "scan", "rank_emit"),
                                             st_last.phase_busy)},
            "plain": plain,
            "autotune": tuned,
            "batched_over_plain": (value / max(1, world)) / plain["tris_per_s"] if plain else None,
            "serving": serve,
            "raster": raster,
            "features": features,
        }
        print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


# -------------------------------------------------------------- serving ----
def feature_frames(ctx, stream, sh, base_ms, frames=10, warmup=3):
    """The 4096-model frame with one vertex-stage feature on for every model (scenes.frame_variant):
    device time per animated frame (CUDA graph replays, CUDA events on the replay stream), visible
    triangles per second, and the time relative to the plain frame."""
    import torch
    from tetra3d_gb300 import scenes
    out = {}
    for kind in scenes.FRAME_VARIANTS:
        sd = scenes.frame_variant(kind)
        sid = ctx.upload(sd)
        try:
            ctx.graph_capture(sid, sd.camera, animate=True)
            ctx.graph_replay(warmup, stream=sh)
            torch.cuda.synchronize()
            v0, _ = ctx.counters()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.graph_replay(frames, stream=sh)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / frames
            v1, _ = ctx.counters()
            vis = (v1 - v0) / frames
            st = ctx.sync()
            # the oracle (the reference's algorithm restated on the CPU) on the same frame, all host
            # threads, its output arrays allocated and touched before the timed render
            from oracle import pyoracle
            threads = os.cpu_count() or 1
            rc = pyoracle.Renderer(sd, sd.camera)
            rc.render(threads=threads)
            c0 = time.perf_counter()
            cpu_vis = rc.render(threads=threads)
            cpu_s = time.perf_counter() - c0
            del rc
            out[kind] = {"ms_per_frame": round(ms, 4), "visible_tris": int(vis), "tris_per_s": vis / (ms / 1e3),
                         "time_vs_plain_frame": round(ms / base_ms, 3),
                         "cpu_baseline": {"value": cpu_vis / cpu_s, "unit": "tris/s", "cores": threads, "kind": "port",
                                          "sample": "the whole frame (static transforms), 1 render"},
                         "phase_busy_us_last_frame": {k: round(float(v), 1) for k, v in zip(
                             ("prep", "vertex", "triangles", "hist", "scan", "rank_emit"), st.phase_busy)}}
        finally:
            ctx.release(sid)
    out["note"] = ("4096-model frame with the feature on every model, animated, CUDA graph replays; "
                   "time_vs_plain_frame = ms / the plain frame's ms; cpu_baseline = the oracle on all host threads")
    return out


def serving_sweep(ctx, rates, seconds, max_requests, seed=7, baseline_requests=1000):
    """Continuous-batching server over 64 resident scenes at Poisson rates; then the same requests
    rendered one request per launch, synchronously (the plain request loop)."""
    from tetra3d_gb300 import serving
    from tetra3d_gb300.runtime import Server
    t0 = time.perf_counter()
    sds, centres = serving.serving_scenes(64)
    gen_s = time.perf_counter() - t0
    sids = [ctx.upload(sd) for sd in sds]
    tris = [sd.total_tris() for sd in sds]
    rng = np.random.Generator(np.random.PCG64(seed))
    slots = 8  # launch slots (host threads building and launching batches concurrently)
    srv = Server(ctx, hbm_budget_bytes=150 << 30, max_batch=64, streams=slots, verify=False)
    out = {"scenes": len(sds), "scene_tris_min": int(min(tris)), "scene_tris_max": int(max(tris)),
           "scene_tris_total": int(sum(tris)), "hbm_budget_gb": 150, "max_batch": 64, "slots": slots,
           "max_pairs_per_batch": 4096,
           "scene_gen_s": round(gen_s, 2), "rates": []}
    try:
        jobs, arr = serving.poisson_requests(rng, sids, sds, centres, 2000.0, 128)  # warm-up
        srv.replay(jobs, arr)
        for rate in rates:
            n = int(min(max_requests, max(200, rate * seconds)))
            jobs, arr = serving.poisson_requests(rng, sids, sds, centres, float(rate), n)
            w0 = time.perf_counter()
            comps = srv.replay(jobs, arr)
            wall = time.perf_counter() - w0
            row = dict(rate_req_s=rate, **serving.latency_summary(comps), wall_s=round(wall, 3))
            out["rates"].append(row)
        # saturation: the last rate's requests all arrive at once (the server's capacity)
        w0 = time.perf_counter()
        comps = srv.replay(jobs, np.zeros(len(jobs)))
        bwall = time.perf_counter() - w0
        out["burst"] = dict(**serving.latency_summary(comps), wall_s=round(bwall, 3))
        # served roofline: the burst's algorithmic bytes over its wall time (all requests queued at
        # once: the server's capacity), against the measured HBM bandwidth
        peak, peak_kind = peaks()
        gbs = out["burst"]["algorithmic_bytes"] / bwall / 1e9
        out["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                           "peak_source": f"{peak_kind} hbm_gbs",
                           "note": "burst of the last rate's requests: algorithmic bytes / wall time incl. host work"}
        # one request per launch, synchronously, over the last rate's requests
        jobs = jobs[:baseline_requests]
        lat, vis = [], 0
        b0 = time.perf_counter()
        for j in jobs:
            s0 = time.perf_counter()
            ctx.render_jobs([j], mode=1)
            vis += int(ctx.sync().visible_tris)
            lat.append((time.perf_counter() - s0) * 1e3)
        el = time.perf_counter() - b0
        out["one_request_per_launch"] = {"requests": len(jobs), "tris_per_s": vis / el, "req_per_s": len(jobs) / el,
                                         "p50_ms": float(np.percentile(lat, 50)),
                                         "p99_ms": float(np.percentile(lat, 99))}
    finally:
        srv.close()
        for s in sids:
            ctx.release(s)
    return out


def run_serving(args, rank, world, local_rank):
    import torch
    import __graft_entry__
    from tetra3d_gb300.runtime import Context
    __graft_entry__.build()
    torch.cuda.set_device(local_rank)
    if rank != 0:
        return
    ctx = Context(local_rank)
    rates = [int(r) for r in args.rates.split(",")]
    with ClockSampler(local_rank) as clk:
        sv = serving_sweep(ctx, rates, args.serve_seconds, args.serve_max_requests)
    top = max(sv["rates"], key=lambda r: r["tris_per_s"])
    line = {"metric": METRIC, "value": top["tris_per_s"], "unit": UNIT, "n_gpus": world, "steps": len(rates),
            "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "serving_64_scenes_poisson", "rates_req_s": rates,
                       "form": "continuous batching server (t3d_server), requests via the C ABI"},
            "serving": sv, "clocks": clk.summary(),
            "e2e": {"value": top["tris_per_s"], "unit": UNIT, "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                    "note": "requests enter through t3d_server_replay from host memory; completions are read back"},
            "served_over_one_request_per_launch": top["tris_per_s"] / sv["one_request_per_launch"]["tris_per_s"],
            "burst_over_one_request_per_launch": sv["burst"]["tris_per_s"] / sv["one_request_per_launch"]["tris_per_s"]}
    print(json.dumps(line))
    ctx.close()


# ------------------------------------------------------------ reference ----
def run_reference(args, rank, world):
    """The reference's path for the same workload, config and metric on the host cores: the
    oracle (Camera.Render restated on the CPU; the Go reference cannot run here) renders
    every model of every frame, frame k with every model's animation step applied k times,
    exactly the frames the GPU arm's graph replays render. Steps are whole frames."""
    if rank != 0:
        return
    sd = make_scene(args.workload, args.models)
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    animate = args.workload == "batched"
    # the output arrays are allocated once, as the reference's render loop reuses its scratch
    r = pyoracle.Renderer(sd, sd.camera)
    for w in range(args.warmup):
        r.render(animate_frames=(w + 1) if animate else 0, threads=threads)
    vis = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        vis += r.render(animate_frames=(args.warmup + k + 1) if animate else 0, threads=threads)
    el = time.perf_counter() - t0
    value = vis / el
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": dict(workload_config(args.workload, sd), form="CPU restatement of Camera.Render",
                           animated=animate),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "cpu_model": cpu_model(), "kind": "port",
                             "sample": f"whole frames ({sd.nmodels} models{', animated' if animate else ''}), "
                                       f"render pairs split over {threads} host threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=240)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "terrain", "cubes", "sphere", "serving"])
    ap.add_argument("--models", type=int, default=4096, help="models in the batched scene (4096 = the full workload)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (default tuning: 2048-triangle "
                                                              "tiles, one launch per phase)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-serving", action="store_true", help="skip the serving sweep in the default run")
    ap.add_argument("--no-raster", action="store_true", help="skip rasterising the last frame")
    ap.add_argument("--no-features", action="store_true",
                    help="skip the frame variants with shape keys, skinning, billboards, subdivision, batching")
    ap.add_argument("--textured", action="store_true",
                    help="texture every material for the raster (three textures, both filters, UV and screen "
                         "mapping, alpha clip on some)")
    ap.add_argument("--rates", default="100,1000,5000,20000", help="serving request rates (req/s)")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival span per serving rate")
    ap.add_argument("--serve-max-requests", type=int, default=8000)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.gpus == 1 else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "serving":
        run_serving(args, rank, world, local_rank)
        return
    run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
