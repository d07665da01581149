"""GPU parity: the CUDA library against the oracle, bit for bit, through the C ABI.

Sizes are reduced so the oracle finishes in seconds; full sizes are covered by
property tests in test_gpu_full.py.
"""
import numpy as np
import pytest

from tetra3d_gb300 import abi, scenes
from oracle import pyoracle
from tests.parity import assert_frames_equal

pytestmark = pytest.mark.gpu

KINDS = ["sphere", "cubes", "terrain", "batched"]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("mode", [abi.MODE_BATCHED, abi.MODE_PLAIN])
def test_small_scenes_match_oracle(ctx, kind, mode):
    sd = scenes.small_variant(kind, seed=11)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera, mode=mode)
        got = ctx.download()
        ref = pyoracle.render(sd, sd.camera)
        assert ref.visible_tris > 0
        assert_frames_equal(got, ref, f"{kind}/mode{mode}")
    finally:
        ctx.release(sid)


def test_uv_sphere_full_config(ctx):
    sd = scenes.uv_sphere_scene(1)
    sid = ctx.upload(sd)
    ctx.render(sid, sd.camera)
    assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), "sphere")
    ctx.release(sid)


def test_cubes_full_config(ctx):
    sd = scenes.cubes_scene(2)
    sid = ctx.upload(sd)
    for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
        ctx.render(sid, sd.camera, mode=mode)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), f"cubes/mode{mode}")
    ctx.release(sid)
