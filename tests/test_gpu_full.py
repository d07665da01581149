"""Full-size workloads on the GPU against the oracle and through size-independent
properties:

- the whole 4096-model frame (69.7 M triangles), static and after three animated
  graph replays, bit for bit against the oracle on all host threads;
- render pairs are independent, so the oracle on a sample of the models (every
  k-th) reproduces those models' pairs inside the full frame;
- the plain form (one launch per pair) and the batched form give identical bits,
  and so do the meshlet and per-vertex record routes and the batched frame as one
  cooperative launch or as one launch per phase;
- a static frame rendered twice gives identical bits (idempotence);
- visible counts add up (segments vs stats vs device counters).
"""
import os

import numpy as np
import pytest

from tetra3d_gb300 import abi, scenes
from oracle import pyoracle
from tests.parity import assert_frames_equal, bits

pytestmark = pytest.mark.gpu


def _pairs(frame):
    out, b = {}, 0
    for s in frame.segments:
        n = s["count"]
        out[(s["model"], s["part"])] = (b, n)
        b += n
    return out


def _check_sample(got, sd, cam, stride, animate_frames=0):
    keep = np.arange(0, sd.nmodels, stride)
    ref = pyoracle.render(scenes.subset(sd, keep), cam, animate_frames=animate_frames, threads=8)
    gp = _pairs(got)
    b = 0
    checked = 0
    for s in ref.segments:
        n = s["count"]
        gb, gn = gp[(int(keep[s["model"]]), s["part"])]
        assert gn == n, f"model {keep[s['model']]} part {s['part']}: {gn} vs oracle {n} triangles"
        for name in ("xyuv", "rgba", "depth"):
            assert np.array_equal(bits(getattr(got, name)[gb:gb + n]), bits(getattr(ref, name)[b:b + n])), \
                f"model {keep[s['model']]} part {s['part']}: {name} differs"
        b += n
        checked += n
    assert checked > 0
    return checked


def test_batched_4096_models(ctx):
    sd = scenes.batched_scene(4)
    cam = sd.camera
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam, mode=abi.MODE_BATCHED)
        st = ctx.sync()
        got = ctx.download(st)
        assert got.visible_tris == sum(s["count"] for s in got.segments) == int(st.visible_tris)
        assert 0 < got.visible_tris < sd.total_tris()
        _check_sample(got, sd, cam, stride=32)
        # plain form: same bits
        ctx.render(sid, cam, mode=abi.MODE_PLAIN)
        plain = ctx.download()
        assert [(s["model"], s["part"], s["count"]) for s in plain.segments] == \
               [(s["model"], s["part"], s["count"]) for s in got.segments]
        for name in ("xyuv", "rgba", "depth"):
            assert np.array_equal(bits(getattr(plain, name)), bits(getattr(got, name))), name
        del plain
        # idempotence of a static frame, and the device counters
        v0, _ = ctx.counters()
        ctx.render(sid, cam, mode=abi.MODE_BATCHED)
        again = ctx.download()
        v1, _ = ctx.counters()
        assert v1 - v0 == got.visible_tris
        for name in ("xyuv", "rgba", "depth"):
            assert np.array_equal(bits(getattr(again, name)), bits(getattr(got, name))), name
    finally:
        ctx.release(sid)


def test_batched_4096_models_animated_graph(ctx):
    sd = scenes.batched_scene(4)
    sid = ctx.upload(sd)
    try:
        ctx.graph_capture(sid, sd.camera, animate=True)
        ctx.graph_replay(3)
        got = ctx.download()
        _check_sample(got, sd, sd.camera, stride=64, animate_frames=3)
    finally:
        ctx.release(sid)


def test_batched_4096_models_whole_frame_matches_oracle(ctx):
    """The benchmarked frame itself, every triangle of every pair: static, then after three
    animated graph replays; and the per-vertex record route gives the same bits."""
    sd = scenes.batched_scene(4)
    threads = os.cpu_count() or 8
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera, mode=abi.MODE_BATCHED)
        got = ctx.download()
        ref = pyoracle.render(sd, sd.camera, threads=threads)
        assert_frames_equal(got, ref, "4096 models, static")
        del ref
        ctx.set_split_phases(0)
        ctx.render(sid, sd.camera, mode=abi.MODE_BATCHED)
        coop = ctx.download()
        assert_frames_equal(coop, got, "one cooperative launch vs one launch per phase")
        del coop
        ctx.set_split_phases(1)
        ctx.set_meshlets(0)
        ctx.render(sid, sd.camera, mode=abi.MODE_BATCHED)
        rec = ctx.download()
        assert_frames_equal(rec, got, "record route vs meshlet route")
        del rec, got
        ctx.set_meshlets(1)
        ctx.graph_capture(sid, sd.camera, animate=True)
        ctx.graph_replay(3)
        got = ctx.download()
        assert_frames_equal(got, pyoracle.render(sd, sd.camera, animate_frames=3, threads=threads),
                            "4096 models, 3 animated replays")
    finally:
        ctx.set_meshlets(1)
        ctx.set_split_phases(1)
        ctx.release(sid)


def test_terrain_full_config(ctx):
    sd = scenes.terrain_scene(3)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera, threads=8), "terrain 1024^2")
    finally:
        ctx.release(sid)
