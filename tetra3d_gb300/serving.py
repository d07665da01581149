"""Serving workload: resident scenes, Poisson render requests, latency statistics.

A request is (scene id, camera pose, resolution, light subset), the render
request of a game server or a remote viewer. The scenes stay resident on the
device; t3d_server admits requests by an HBM budget and batches those waiting
into one launch per free slot (continuous batching, csrc/t3d_serve.cu).
"""
import math

import numpy as np

from . import abi, scenes
from .runtime import job

F32 = np.float32
RESOLUTIONS = [(640, 360), (1280, 720), (1920, 1080)]


def serving_scenes(n=64, seed=100):
    """n scenes drawn from the sphere, cubes and terrain workloads with varied seeds and sizes
    (about 1k to 2.1M triangles each). Returns (scenes, centres)."""
    out, centres = [], []
    for i in range(n):
        s = seed + i
        k = i % 8
        if k in (0, 4):
            sd = scenes.uv_sphere_scene(s)                      # 960 triangles
            c = (0.0, 0.0, -5.0)
        elif k in (1, 5):
            sd = scenes.cubes_scene(s, n=1000 if k == 1 else 250)  # 12k / 3k triangles
            c = (0.0, 0.0, 0.0)
        elif k in (2, 6):
            sd = scenes.terrain_scene(s, n=256 if k == 2 else 512, extent=100.0)  # 130k / 522k triangles
            c = (0.0, 0.0, 0.0)
        elif k == 3:
            sd = scenes.small_variant("batched", s)             # 48 models, ~50k triangles
            c = (0.0, 0.0, 60.0)
        else:
            sd = scenes.terrain_scene(s, n=1024 if i % 16 == 7 else 512)  # 2.09M / 522k triangles
            c = (0.0, 0.0, 0.0)
        out.append(sd)
        centres.append(np.asarray(c, F32))
    return out, centres


def random_camera(rng, centre):
    """A camera on a sphere of radius 10-100 around `centre`, looking at it, at a random resolution."""
    r = rng.uniform(10.0, 100.0)
    z = rng.uniform(-1.0, 1.0)
    phi = rng.uniform(0.0, 2.0 * math.pi)
    d = np.array([math.sqrt(1 - z * z) * math.cos(phi), z, math.sqrt(1 - z * z) * math.sin(phi)], F32)
    pos = (centre + F32(r) * d).astype(F32)
    rot = scenes.look_rotation(scenes.unit3((pos - centre).astype(F32)))  # the camera looks down -Z
    w, h = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
    return scenes.camera(pos=pos, rot=rot, w=w, h=h, fov=60.0, near=0.1, far=float(2.5 * r + 150.0))


def random_light_mask(rng, nlights):
    """A random subset of the scene's lights (each kept with probability 1/2)."""
    keep = rng.random(nlights) < 0.5
    m = 0
    for i in np.nonzero(keep)[0]:
        m |= 1 << int(i)
    return m


def poisson_requests(rng, scene_ids, sds, centres, rate, count):
    """count requests with exponential inter-arrival times at `rate` per second.
    Returns (jobs, arrival seconds)."""
    gaps = rng.exponential(1.0 / rate, count)
    arrivals = np.cumsum(gaps) - gaps[0]
    jobs = []
    for _ in range(count):
        s = int(rng.integers(len(scene_ids)))
        cam = random_camera(rng, centres[s])
        jobs.append(job(scene_ids[s], cam, random_light_mask(rng, sds[s].nlights)))
    return jobs, arrivals


def latency_summary(completions):
    """p50/p99/max latency (ms, done - arrival), triangles/s over the span, statuses."""
    ok = [c for c in completions if c.status == abi.T3D_OK]
    lat = np.array([(c.done_s - c.arrival_s) * 1e3 for c in ok]) if ok else np.zeros(1)
    span = (max(c.done_s for c in ok) - min(c.arrival_s for c in ok)) if ok else 0.0
    tris = sum(int(c.visible_tris) for c in ok)
    # algorithmic bytes (48V+12T+64+48L of surviving models + 108 per visible triangle)
    alg = sum(int(c.model_bytes) + 108 * int(c.visible_tris) for c in ok)
    # where the time goes: queue wait (arrival -> admission), launch-table build and launch
    # (admission -> launch), device work and read-back (launch -> completion)
    def pct(v, q):
        return float(np.percentile(v, q)) if len(v) else 0.0
    wait = [(c.admit_s - c.arrival_s) * 1e3 for c in ok]
    build = [(c.launch_s - c.admit_s) * 1e3 for c in ok]
    dev = [(c.done_s - c.launch_s) * 1e3 for c in ok]
    return {"requests": len(completions), "ok": len(ok), "algorithmic_bytes": alg,
            "algorithmic_gb_per_s": alg / span / 1e9 if span > 0 else 0.0,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(lat.max()), "tris_per_s": tris / span if span > 0 else 0.0,
            "req_per_s": len(ok) / span if span > 0 else 0.0, "visible_tris": tris,
            "mean_batch": float(np.mean([c.batch for c in ok])) if ok else 0.0,
            "wait_ms_p50_p99": [pct(wait, 50), pct(wait, 99)],
            "build_ms_p50_p99": [pct(build, 50), pct(build, 99)],
            "device_ms_p50_p99": [pct(dev, 50), pct(dev, 99)]}
