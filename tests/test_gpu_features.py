"""GPU vs oracle, bit for bit, through the C ABI, over every option of the stage:
material / model / light options (feature scenes) under every camera option, both
forms; several jobs with light masks in one launch; animation inside the launch and
through CUDA graph replay; transform read-back; serving (same bits alone and in a
mix); argument errors."""
import ctypes as C
import os
import time

import numpy as np
import pytest

from tetra3d_gb300 import abi, scenes
from tetra3d_gb300.runtime import Server, job
from oracle import pyoracle
from tests.parity import assert_frames_equal, bits

pytestmark = pytest.mark.gpu


# batched as one launch per phase (the default), batched as one cooperative launch, plain
FORMS = [(abi.MODE_BATCHED, 1), (abi.MODE_BATCHED, 0), (abi.MODE_PLAIN, 1)]


@pytest.mark.parametrize("variant", scenes.FEATURE_CAMERAS)
@pytest.mark.parametrize("mode,split", FORMS)
def test_feature_scenes_match_oracle(ctx, variant, mode, split):
    for seed in (5, 6):
        sd = scenes.feature_scene(seed)
        cam = scenes.feature_camera(variant)
        sid = ctx.upload(sd)
        try:
            ctx.set_split_phases(split)
            ctx.render(sid, cam, mode=mode)
            got = ctx.download()
        finally:
            ctx.set_split_phases(1)
            ctx.release(sid)
        ref = pyoracle.render(sd, cam)
        assert ref.visible_tris > 0
        assert_frames_equal(got, ref, f"features{seed}/{variant}/mode{mode}/split{split}")


class _JobFrame:
    def __init__(self, segments, xyuv, rgba, depth):
        self.segments, self.xyuv, self.rgba, self.depth = segments, xyuv, rgba, depth
        self.visible_tris = int(xyuv.shape[0])


def split_jobs(frame, njobs):
    """Per-job views of a multi-job download (compacted in segment order)."""
    out, b = [], 0
    per = [[] for _ in range(njobs)]
    for s in frame.segments:
        per[s["job"]].append((s, b))
        b += s["count"]
    for j in range(njobs):
        idx = np.concatenate([np.arange(b0, b0 + s["count"]) for s, b0 in per[j]] or [np.zeros(0, np.int64)])
        idx = idx.astype(np.int64)
        out.append(_JobFrame([s for s, _ in per[j]], frame.xyuv[idx], frame.rgba[idx], frame.depth[idx]))
    return out


def test_jobs_with_light_masks_in_one_launch(ctx):
    a = scenes.feature_scene(5)
    b = scenes.small_variant("batched", 12)
    sa, sb = ctx.upload(a), ctx.upload(b)
    try:
        specs = [(sa, a, scenes.feature_camera("persp"), None),
                 (sa, a, scenes.feature_camera("tilted"), ((1 << 128) - 1) & ~((1 << 1) | (1 << 6))),
                 (sb, b, scenes.feature_camera("fog_sub"), ((1 << 128) - 1) & ~(1 << 3)),
                 (sb, b, b.camera, None)]
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render_jobs([job(s, cam, mask) for s, _, cam, mask in specs], mode=mode)
            parts = split_jobs(ctx.download(), len(specs))
            for j, (s, sd, cam, mask) in enumerate(specs):
                assert_frames_equal(parts[j], pyoracle.render(sd, cam, light_mask=mask), f"job{j}/mode{mode}")
    finally:
        ctx.release(sa)
        ctx.release(sb)


def _host_transforms(sd, k):
    n = sd.nmodels
    rot = sd.mv["rotation"].reshape(n, 4, 4).copy()
    step = sd.mv["rotate_step"].reshape(n, 4, 4)
    for _ in range(k):
        rot = scenes.mult(step, rot)
    return scenes.trs(sd.mv["position"], sd.mv["scale"], rot)


def test_animation_in_launch_matches_oracle(ctx):
    sd = scenes.small_variant("batched", 8)
    sid = ctx.upload(sd)
    try:
        for k in (1, 2, 3):
            ctx.render(sid, sd.camera, mode=abi.MODE_BATCHED, animate=True)
            assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera, animate_frames=k), f"animate {k}")
        T = ctx.transforms(sid, sd.nmodels)
        assert np.array_equal(bits(T), bits(_host_transforms(sd, 3)))
    finally:
        ctx.release(sid)


def test_graph_replay_matches_oracle(ctx):
    sd = scenes.small_variant("batched", 9)
    sid = ctx.upload(sd)
    try:
        ctx.graph_capture(sid, sd.camera, animate=True)
        ctx.graph_replay(4)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera, animate_frames=4), "graph x4")
        ctx.graph_replay(1)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera, animate_frames=5), "graph x5")
        assert np.array_equal(bits(ctx.transforms(sid, sd.nmodels)), bits(_host_transforms(sd, 5)))
        # static capture: replays give the same frame every time
        ctx.set_models(sid, sd)
        ctx.graph_capture(sid, sd.camera, animate=False)
        ctx.graph_replay(3)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), "static graph")
    finally:
        ctx.release(sid)


def test_set_models_between_frames(ctx):
    sd = scenes.feature_scene(6)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera)
        ctx.sync()
        sd.mv["position"][:, 0] += np.float32(1.5)
        sd.mv["transform"] = scenes.trs(sd.mv["position"], sd.mv["scale"],
                                        sd.mv["rotation"].reshape(-1, 4, 4)).reshape(-1, 16)
        ctx.set_models(sid, sd, first=4, n=sd.nmodels - 4)  # the first four keep their old place
        moved = scenes.feature_scene(6)
        moved.mv[4:] = sd.mv[4:]
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), pyoracle.render(moved, sd.camera), "partial set_models")
    finally:
        ctx.release(sid)


def _fnv_frame(f):
    """FNV-1a over xyuv, rgba, depth bytes of each segment in emit order (the server's checksum)."""
    h = 1469598103934665603
    b = 0
    for s in f.segments:
        n = s["count"]
        if not n:
            continue
        for arr in (f.xyuv[b:b + n], f.rgba[b:b + n], f.depth[b:b + n]):
            for byte in np.ascontiguousarray(arr, np.float32).tobytes():
                h = ((h ^ byte) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
        b += n
    return h


def _drain(srv, n, timeout=60.0):
    got, t0 = {}, time.time()
    while len(got) < n and time.time() - t0 < timeout:
        for c in srv.poll():
            got[c.id] = c
        time.sleep(0.002)
    assert len(got) == n, f"{len(got)} of {n} completions"
    return got


def test_serving_same_bits_alone_and_in_mix(ctx):
    sds = [scenes.feature_scene(s) for s in (5, 6, 7)] + [scenes.small_variant("batched", 13)]
    sids = [ctx.upload(sd) for sd in sds]
    cams = [scenes.feature_camera(v) for v in ("persp", "tilted", "fog_add", "ortho")]
    reqs = [(i, sids[i % 4], sds[i % 4], cams[(i // 4) % 4]) for i in range(12)]
    srv = Server(ctx, hbm_budget_bytes=8 << 30, max_batch=8, streams=2, verify=True)
    try:
        alone = {}
        for rid, sid, sd, cam in reqs:
            assert srv.submit(job(sid, cam), rid) == abi.T3D_OK
            c = _drain(srv, 1)[rid]
            assert c.status == abi.T3D_OK
            alone[rid] = (c.checksum, c.visible_tris)
        for rid, sid, sd, cam in reqs:
            assert srv.submit(job(sid, cam), 100 + rid) == abi.T3D_OK
        mix = _drain(srv, len(reqs))
        for rid, sid, sd, cam in reqs:
            c = mix[100 + rid]
            assert c.status == abi.T3D_OK
            assert (c.checksum, c.visible_tris) == alone[rid], f"request {rid} differs in the mix"
            assert c.admit_s >= c.arrival_s and c.done_s >= c.launch_s >= c.admit_s and c.batch >= 1
        # a bound of one render pair per batch: every request goes alone, with the same bits
        ctx.lib.t3d_server_set_batch_pairs(srv.h, 1)
        for rid, sid, sd, cam in reqs:
            assert srv.submit(job(sid, cam), 200 + rid) == abi.T3D_OK
        one = _drain(srv, len(reqs))
        for rid, sid, sd, cam in reqs:
            c = one[200 + rid]
            assert c.status == abi.T3D_OK and c.batch == 1
            assert (c.checksum, c.visible_tris) == alone[rid], f"request {rid} differs batched alone"
        for rid, sid, sd, cam in reqs[:4]:  # the checksum is over the oracle's bits
            ref = pyoracle.render(sd, cam)
            assert alone[rid] == (_fnv_frame(ref), ref.visible_tris)
    finally:
        srv.close()
        for s in sids:
            ctx.release(s)


def test_serving_scenes_match_oracle_alone_and_in_mix(ctx):
    """The serving workload's own scenes (sphere, 1000 and 250 cubes, 256^2 / 512^2 / 1024^2
    terrains, the 48-model batched scene), random cameras on the 10-100 sphere at the three
    resolutions and random light subsets: every request's stream alone and in the mix equals
    the oracle's."""
    from tetra3d_gb300 import serving
    sds, centres = serving.serving_scenes(n=8)
    sids = [ctx.upload(sd) for sd in sds]
    rng = np.random.Generator(np.random.PCG64(77))
    reqs = []
    for rid in range(16):
        s = rid % 8
        reqs.append((rid, s, serving.random_camera(rng, centres[s]), serving.random_light_mask(rng, sds[s].nlights)))
    assert {(c.width, c.height) for _, _, c, _ in reqs} == set(serving.RESOLUTIONS)
    srv = Server(ctx, hbm_budget_bytes=32 << 30, max_batch=8, streams=2, verify=True)
    try:
        alone = {}
        for rid, s, cam, mask in reqs:
            assert srv.submit(job(sids[s], cam, mask), rid) == abi.T3D_OK
            c = _drain(srv, 1)[rid]
            assert c.status == abi.T3D_OK
            alone[rid] = (c.checksum, c.visible_tris)
        for rid, s, cam, mask in reqs:
            assert srv.submit(job(sids[s], cam, mask), 100 + rid) == abi.T3D_OK
        mix = _drain(srv, len(reqs))
        for rid, s, cam, mask in reqs:
            c = mix[100 + rid]
            assert c.status == abi.T3D_OK
            assert (c.checksum, c.visible_tris) == alone[rid], f"request {rid} differs in the mix"
            ref = pyoracle.render(sds[s], cam, light_mask=mask, threads=8)
            assert alone[rid] == (_fnv_frame(ref), ref.visible_tris), f"request {rid} (scene {s}) differs from the oracle"
    finally:
        srv.close()
        for sid in sids:
            ctx.release(sid)


def test_serving_admission(ctx):
    sd = scenes.small_variant("batched", 14)
    sid = ctx.upload(sd)
    srv = Server(ctx, hbm_budget_bytes=1 << 10, max_batch=4, streams=1, verify=False)
    try:
        assert srv.submit(job(sid, sd.camera), 1) == abi.T3D_E_ADMIT  # larger than the whole budget
        assert srv.submit(job(12345, sd.camera), 2) == abi.T3D_E_NOTFOUND
    finally:
        srv.close()
        ctx.release(sid)


def test_argument_errors(ctx):
    lib = ctx.lib
    sd = scenes.uv_sphere_scene(1)
    sid = ctx.upload(sd)
    try:
        assert lib.t3d_scene_release(ctx.h, 999999) == abi.T3D_E_NOTFOUND
        assert lib.t3d_render(ctx.h, 999999, C.byref(sd.camera), abi.MODE_BATCHED, 0, None) == abi.T3D_E_NOTFOUND
        assert lib.t3d_render(ctx.h, sid, C.byref(sd.camera), 7, 0, None) == abi.T3D_E_INVAL
        j = (abi.JobDesc * 2)(job(sid, sd.camera), job(sid, sd.camera))
        assert lib.t3d_render_jobs(ctx.h, j, 2, abi.MODE_BATCHED, 1, None) == abi.T3D_E_INVAL  # animate twice
        fresh = C.c_void_p()
        assert lib.t3d_create(0, C.byref(fresh)) == abi.T3D_OK
        assert lib.t3d_graph_replay(fresh, 1, None) == abi.T3D_E_INVAL
        lib.t3d_destroy(fresh)
        bad = scenes.uv_sphere_scene(1)
        bad.mv["mesh"][0] = 5
        d = bad.desc()
        out = C.c_uint32()
        assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
        assert b"mesh" in lib.t3d_last_error(ctx.h)
        bad = scenes.uv_sphere_scene(1)
        bad.meshes[0].parts[0]["mat"]["sort_mode"] = 9
        d = bad.desc()
        assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
        bad = scenes.uv_sphere_scene(1)
        bad.meshes[0].indices[3, 1] = bad.meshes[0].nverts  # index past the vertex array
        d = bad.desc()
        assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
        bad = scenes.uv_sphere_scene(1)
        bad.mv["light_list"][0] = 3
        d = bad.desc()
        assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
        # the context still works after rejected calls
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), "after errors")
    finally:
        ctx.release(sid)


def test_reused_launch_tables_follow_model_updates(ctx):
    """Renders that change only transforms of an opaque scene reuse the launch tables; changes
    that alter the tables (colour -> transparency, visibility) rebuild them. Every frame must
    match the oracle."""
    sd = scenes.small_variant("batched", 15)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), "first")
        n = sd.nmodels
        for k in range(3):  # transforms only: tables reused
            rot = scenes.mult(sd.mv["rotate_step"].reshape(n, 4, 4), sd.mv["rotation"].reshape(n, 4, 4))
            sd.mv["rotation"] = rot.reshape(n, 16)
            sd.mv["position"][:, 1] += np.float32(0.25)
            sd.mv["transform"] = scenes.trs(sd.mv["position"], sd.mv["scale"], rot).reshape(n, 16)
            sd.mv["world_rotation"] = rot.reshape(n, 16)
            ctx.set_models(sid, sd)
            ctx.render(sid, sd.camera)
            st = ctx.sync()
            assert st.h2d_bytes == 0, "launch tables were rebuilt for a transform-only update"
            assert_frames_equal(ctx.download(st), pyoracle.render(sd, sd.camera), f"transforms {k}")
        sd.mv["color"][::3, 3] = np.float32(0.5)   # some models become transparent
        sd.mv["visible"][1] = 0
        ctx.set_models(sid, sd)
        ctx.render(sid, sd.camera)
        st = ctx.sync()
        assert st.h2d_bytes > 0
        assert_frames_equal(ctx.download(st), pyoracle.render(sd, sd.camera), "structure change")
        sd.mv["position"][:, 0] -= np.float32(0.5)  # transparents present: the draw order follows transforms
        sd.mv["transform"] = scenes.trs(sd.mv["position"], sd.mv["scale"],
                                        sd.mv["rotation"].reshape(n, 4, 4)).reshape(n, 16)
        ctx.set_models(sid, sd)
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), "transparent reorder")
    finally:
        ctx.release(sid)


def _max_light_scene(nlights, seed=21):
    sd = scenes.batched_scene(seed, n=24, vmin=24, vmax=1500, nlights=nlights, box=40.0, max_levels=3)
    sd.mv["light_list"] = -1
    return sd


@pytest.mark.parametrize("mixed", [False, True])
def test_max_light_count_matches_oracle(ctx, mixed):
    """Camera.MaxLightCount on the device path against the oracle; `mixed` adds extra ambient and
    directional lights, where the reference's comparator is not a strict order and the result is
    that of Go's stable sort algorithm."""
    sd = _max_light_scene(40)
    if mixed:
        for i in (7, 19, 33):
            sd.lights[i].type = abi.LIGHT_DIRECTIONAL
        sd.lights[25].type = abi.LIGHT_AMBIENT
    for keep, focus in ((25, None), (30, (10.0, -5.0, 20.0)), (3, None)):
        cam = sd.camera
        cam.max_light_count = keep
        cam.focus_set = int(focus is not None)
        if focus is not None:
            cam.focus[:] = list(focus)
        sid = ctx.upload(sd)
        try:
            ctx.render(sid, cam)
            assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), f"keep {keep} mixed {mixed}")
        finally:
            ctx.release(sid)


@pytest.mark.parametrize("variant", scenes.FEATURE_CAMERAS)
def test_skinned_scene_matches_oracle(ctx, variant):
    """Skinned models (bone blends, a 1.0 weight after a partial one), shape keys on skinned and
    unskinned meshes, skinned meshes drawn unskinned, under every light and material option."""
    sd = scenes.skinned_scene(7)
    cam = scenes.feature_camera(variant)
    ref = pyoracle.render(sd, cam)
    assert ref.visible_tris > 0
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            assert_frames_equal(ctx.download(), ref, f"skinned/{variant}/mode{mode}")
    finally:
        ctx.release(sid)


def test_bones_and_shape_weights_between_frames(ctx):
    """New bone influences (all, then a sub-range) and shape-key weights between frames."""
    sd = scenes.skinned_scene(8)
    cam = scenes.feature_camera("persp")
    nskin = int(sd.mv["skinned"].sum())
    rng = np.random.default_rng(11)
    pos = sd.mv["position"][:nskin, :3]
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), "initial")
        sd.bones = scenes.tube_bones(rng, nskin, pos, bend=0.9)
        ctx.set_bones(sid, sd.bones)
        sd.meshes[3].shape_weights = np.array([0.2, 0.9], np.float32)
        ctx.set_shape_weights(sid, 3, sd.meshes[3].shape_weights)
        ctx.render(sid, cam)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), "new bones and weights")
        part = scenes.tube_bones(rng, 2, pos[2:4], bend=1.2)
        sd.bones = sd.bones.copy()
        sd.bones[8:16] = part
        ctx.set_bones(sid, part, first=8)
        sd.meshes[2].shape_weights = np.array([-0.4], np.float32)
        ctx.set_shape_weights(sid, 2, sd.meshes[2].shape_weights)
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), f"bone range, mode{mode}")
    finally:
        ctx.release(sid)


def test_skinning_argument_errors(ctx):
    lib = ctx.lib
    sd = scenes.skinned_scene(7)
    out = C.c_uint32()
    bad = scenes.skinned_scene(7)
    bad.mv["bone_first"][3] = bad.bones.shape[0] - 2  # joints 2, 3 past the last bone
    d = bad.desc()
    assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
    assert b"bone" in lib.t3d_last_error(ctx.h)
    bad = scenes.skinned_scene(7)
    bad.mv["skinned"][20] = 1
    bad.mv["mesh"][20] = 4  # the cube has no joints
    d = bad.desc()
    assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
    sid = ctx.upload(sd)
    try:
        b = np.zeros((3, 16), np.float32)
        nb = sd.bones.shape[0]
        assert lib.t3d_scene_set_bones(ctx.h, sid, nb - 2, abi.fptr(b), 3) == abi.T3D_E_INVAL
        w = np.zeros(3, np.float32)
        assert lib.t3d_scene_set_shape_weights(ctx.h, sid, 3, abi.fptr(w), 3) == abi.T3D_E_INVAL
        assert lib.t3d_scene_set_shape_weights(ctx.h, sid, 9, abi.fptr(w), 2) == abi.T3D_E_INVAL
        m = (abi.ModelDesc * 1)(sd.models[5])
        m[0].bone_first = nb
        assert lib.t3d_scene_set_models(ctx.h, sid, 5, m, 1) == abi.T3D_E_INVAL
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), "after errors")
    finally:
        ctx.release(sid)


@pytest.mark.parametrize("variant", scenes.FEATURE_CAMERAS + ["down"])
def test_billboard_scene_matches_oracle(ctx, variant):
    """Billboarded parts under every lock / up direction / depth mode, a LookAt straight up
    (the `down` camera), a billboard material on a skinned model, in both forms."""
    sd = scenes.billboard_scene(9)
    cam = scenes.down_camera() if variant == "down" else scenes.feature_camera(variant)
    ref = pyoracle.render(sd, cam)
    assert ref.visible_tris > 0
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            assert_frames_equal(ctx.download(), ref, f"billboards/{variant}/mode{mode}")
    finally:
        ctx.release(sid)


@pytest.mark.parametrize("variant", ["persp", "ortho", "tilted", "fog_add", "unlit"])
def test_subdivision_scene_matches_oracle(ctx, variant):
    """Auto-subdivided meshes: per-frame level choice per triangle (closest point on the
    triangle to the model-space camera), subdivided vertices and centres, both forms."""
    sd = scenes.subdivision_scene(10)
    cam = scenes.feature_camera(variant)
    ref = pyoracle.render(sd, cam)
    assert ref.visible_tris > 0
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            assert_frames_equal(ctx.download(), ref, f"subdivision/{variant}/mode{mode}")
        # the camera moves: triangles change level
        for step in range(3):
            cam2 = scenes.camera(pos=(0.0, 0.5, -4.0 - 8.0 * step), w=1280, h=720, fov=65.0, near=0.1, far=60.0)
            ctx.render(sid, cam2)
            assert_frames_equal(ctx.download(), pyoracle.render(sd, cam2), f"subdivision/moved{step}")
    finally:
        ctx.release(sid)


def test_subdivision_argument_errors(ctx):
    lib = ctx.lib
    out = C.c_uint32()
    bad = scenes.subdivision_scene(10)
    bad.subdivision_levels = np.array([(36.0, 0.0)], np.float32)  # the level loop would not end
    d = bad.desc()
    assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
    bad = scenes.subdivision_scene(10)
    bad.meshes[0].shape_positions = np.zeros((1, bad.meshes[0].nverts, 3), np.float32)
    bad.meshes[0].shape_normals = np.zeros((1, bad.meshes[0].nverts, 3), np.float32)
    bad.meshes[0].shape_weights = np.ones(1, np.float32)
    d = bad.desc()
    assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL
    bad = scenes.subdivision_scene(10)
    bad.max_subdivisions = 9
    d = bad.desc()
    assert lib.t3d_scene_upload(ctx.h, C.byref(d), C.byref(out)) == abi.T3D_E_INVAL


@pytest.mark.parametrize("variant", ["persp", "ortho", "fog_sub"])
def test_vertex_snapping_matches_oracle(ctx, variant):
    """Camera.VertexSnapping on the feature and billboard scenes, both forms."""
    for sd in (scenes.feature_scene(5), scenes.billboard_scene(9)):
        cam = scenes.feature_camera(variant)
        cam.vertex_snapping = 8.0
        ref = pyoracle.render(sd, cam)
        sid = ctx.upload(sd)
        try:
            for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
                ctx.render(sid, cam, mode=mode)
                assert_frames_equal(ctx.download(), ref, f"snap/{sd.name}/{variant}/mode{mode}")
        finally:
            ctx.release(sid)


def test_set_lights_between_frames(ctx):
    """Lights moved, recoloured, re-ranged and switched off (energy 0) between frames, with and
    without MaxLightCount; the launch tables are rebuilt and every frame matches the oracle."""
    sd = scenes.feature_scene(6)
    cam = scenes.feature_camera("persp")
    rng = np.random.default_rng(5)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), "initial")
        for step in range(3):
            first = 1 if step == 1 else 0  # step 1 pushes (and changes) lights 1.. only
            for i in range(first, sd.nlights):
                L = sd.lights[i]
                if L.type == abi.LIGHT_POINT:
                    L.transform[12] += float(rng.uniform(-3, 3))
                    L.transform[14] += float(rng.uniform(-3, 3))
                    L.range = float(rng.uniform(5, 25))
                L.color[0] = float(rng.uniform(0.2, 1.0))
                L.energy = float(rng.uniform(0.0, 2.0)) if step < 2 else 0.0
            ctx.set_lights(sid, sd, first=first, n=sd.nlights - first)
            cam.max_light_count = 4 if step == 1 else 0
            ctx.render(sid, cam)
            assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), f"lights step {step}")
        bad = (abi.LightDesc * 1)(sd.lights[0])
        bad[0].type = 7
        assert ctx.lib.t3d_scene_set_lights(ctx.h, sid, 0, bad, 1) == abi.T3D_E_INVAL
        assert ctx.lib.t3d_scene_set_lights(ctx.h, sid, sd.nlights, bad, 1) == abi.T3D_E_INVAL
    finally:
        ctx.release(sid)


@pytest.mark.parametrize("variant", ["persp", "tilted", "ortho", "fog_add"])
def test_dynamic_batches_match_oracle(ctx, variant):
    """Dynamic batches: members far to near inside their owner's place in the draw order, every
    part, culled members, a nested owner, a transparent batch; the flush numbers of the pairs
    (t3d_segment_info.draw) equal the oracle's."""
    sd = scenes.batch_scene(11)
    cam = scenes.feature_camera(variant)
    ref = pyoracle.render(sd, cam)
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            got = ctx.download()
            assert_frames_equal(got, ref, f"batches/{variant}/mode{mode}")
            assert [(s["draw"], s["draw_transparent"]) for s in got.segments] == \
                   [(s["draw"], s["draw_transparent"]) for s in ref.segments]
        # members moved between frames: the order inside the batches follows
        rng = np.random.default_rng(3)
        sd.mv["position"][3:] += rng.uniform(-4, 4, (sd.nmodels - 3, 3)).astype(np.float32)
        n = sd.nmodels
        sd.mv["transform"] = scenes.trs(sd.mv["position"], sd.mv["scale"],
                                        sd.mv["rotation"].reshape(n, 4, 4)).reshape(n, 16)
        ctx.set_models(sid, sd)
        ctx.render(sid, cam)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), f"batches/{variant}/moved")
    finally:
        ctx.release(sid)


@pytest.mark.parametrize("variant", ["persp", "tilted", "fog_add", "corrected"])
def test_cell_use_lights_match_oracle(ctx, variant):
    """LightVolumeCell.useLights: lights applied to vertices inside light-volume cells, for
    models lit by the scene list and by light groups, both forms; a used light cannot be
    turned into a volume."""
    sd = scenes.nested_light_scene(5)
    cam = scenes.feature_camera(variant)
    ref = pyoracle.render(sd, cam)
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            assert_frames_equal(ctx.download(), ref, f"nested/{variant}/mode{mode}")
        used = sorted({x for c in sd.cell_uses for x in c})
        bad = (abi.LightDesc * 1)(sd.lights[used[0]])
        bad[0].type = abi.LIGHT_VOLUME
        assert ctx.lib.t3d_scene_set_lights(ctx.h, sid, used[0], bad, 1) == abi.T3D_E_INVAL
    finally:
        ctx.release(sid)


def test_all_features_in_one_launch(ctx):
    """Skinned, shape-keyed, billboarded, auto-subdivided, dynamically batched and cell-lit
    scenes as four jobs of one batched launch (with light masks, MaxLightCount and vertex
    snapping on some), and the same jobs one launch per pair: every job bit-exact."""
    sk, bb = scenes.skinned_scene(7), scenes.billboard_scene(9)
    sub, bat = scenes.subdivision_scene(10), scenes.batch_scene(11)
    nested = scenes.nested_light_scene(6)
    ids = [ctx.upload(x) for x in (sk, bb, sub, bat, nested)]
    try:
        c0 = scenes.feature_camera("tilted")
        c1 = scenes.feature_camera("persp")
        c1.vertex_snapping = 16.0
        c2 = scenes.feature_camera("fog_sub")
        c3 = scenes.feature_camera("persp")
        c3.max_light_count = 3
        c4 = scenes.feature_camera("ortho")
        specs = [(ids[0], sk, c0, None), (ids[1], bb, c1, ((1 << 128) - 1) & ~(1 << 2)),
                 (ids[2], sub, c2, None), (ids[3], bat, c3, None), (ids[4], nested, c4, ((1 << 128) - 1) & ~(1 << 1))]
        for mode, split in FORMS:
            ctx.set_split_phases(split)
            ctx.render_jobs([job(s, cam, mask) for s, _, cam, mask in specs], mode=mode)
            parts = split_jobs(ctx.download(), len(specs))
            for j, (s, sd, cam, mask) in enumerate(specs):
                assert_frames_equal(parts[j], pyoracle.render(sd, cam, light_mask=mask),
                                    f"job{j}/mode{mode}/split{split}")
    finally:
        ctx.set_split_phases(1)
        for s in ids:
            ctx.release(s)


def test_graph_replay_follows_bone_updates(ctx):
    """A captured frame of a skinned scene replayed after new bone influences: the graph reads
    the bones from the device, so each replay matches the oracle with the current bones."""
    sd = scenes.skinned_scene(8)
    cam = scenes.feature_camera("persp")
    nskin = int(sd.mv["skinned"].sum())
    pos = sd.mv["position"][:nskin, :3]
    rng = np.random.default_rng(21)
    sid = ctx.upload(sd)
    try:
        ctx.graph_capture(sid, cam, animate=False)
        for k in range(2):
            ctx.graph_replay(1)
            assert_frames_equal(ctx.download(), pyoracle.render(sd, cam), f"replay {k}")
            sd.bones = scenes.tube_bones(rng, nskin, pos, bend=0.7)
            ctx.set_bones(sid, sd.bones)
    finally:
        ctx.release(sid)


def test_edge_cases_match_oracle(ctx):
    """Empty and degenerate inputs: a scene without models, a frame where every model is culled,
    a part with no triangles next to a one-triangle mesh, and a lit scene without lights."""
    cam = scenes.feature_camera("persp")
    # no models at all
    empty = scenes.SceneData([scenes.cube_mesh()], 0, [], [[]], name="empty")
    sid = ctx.upload(empty)
    try:
        ctx.render(sid, cam)
        st = ctx.sync()
        assert st.visible_tris == 0
        assert ctx.download().visible_tris == 0
    finally:
        ctx.release(sid)
    # every model behind the camera
    sd = scenes.feature_scene(5)
    sd.mv["position"][:, 2] = 80.0
    n = sd.nmodels
    sd.mv["transform"] = scenes.trs(sd.mv["position"], sd.mv["scale"], sd.mv["rotation"].reshape(n, 4, 4)).reshape(n, 16)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam)
        got = ctx.download()
        ref = pyoracle.render(sd, cam)
        assert ref.visible_tris == 0
        assert_frames_equal(got, ref, "all culled")
    finally:
        ctx.release(sid)
    # an empty part and a single triangle, lit by an empty light list
    tri = scenes.MeshData(np.array([(-1, -1, 0), (1, -1, 0), (0, 1, 0)], np.float32),
                          np.tile(np.array([0, 0, 1], np.float32), (3, 1)), np.zeros((3, 2), np.float32),
                          np.array([(0, 1, 2)], np.uint32))
    cube = scenes.cube_mesh()
    cube.parts = [dict(tri_start=0, tri_count=0, mat=scenes.default_material()),
                  dict(tri_start=0, tri_count=12, mat=scenes.default_material(backface_culling=0))]
    sd = scenes.SceneData([tri, cube], 2, [], [[]], name="degenerate")
    scenes.set_models_trs(sd, [0, 1], np.array([(0, 0, -4), (2, 0, -6)], np.float32), np.ones((2, 3), np.float32),
                          scenes.ident(2))
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            ref = pyoracle.render(sd, cam)
            assert ref.visible_tris > 0
            assert_frames_equal(ctx.download(), ref, f"degenerate/mode{mode}")
    finally:
        ctx.release(sid)


def test_multi_tile_altered_parts(ctx):
    """Skinned, shape-keyed, billboarded and auto-subdivided parts large enough to span several
    triangle tiles: their tiles go through the histogram / scan / rank phases like plain ones."""
    rng = np.random.default_rng(31)
    tube = scenes.tube_mesh(rings=120, segments=40, height=3.0)
    tube.parts = [dict(tri_start=0, tri_count=tube.ntris, mat=scenes.default_material(backface_culling=0))]
    tube.joints, tube.weights = scenes.tube_skin(tube, rng, 4)
    tube.shape_positions = (0.05 * rng.standard_normal((1, tube.nverts, 3))).astype(np.float32)
    tube.shape_normals = (0.05 * rng.standard_normal((1, tube.nverts, 3))).astype(np.float32)
    tube.shape_weights = np.array([0.5], np.float32)
    grid = scenes.grid_mesh(40, 40, 8.0, 8.0, lambda X, Z: 0.3 * np.sin(X) * np.cos(Z), x0=-4.0, z0=-4.0)
    grid.parts = [dict(tri_start=0, tri_count=grid.ntris, mat=scenes.default_material(backface_culling=0))]
    grid.auto_subdivide = 1
    bb = scenes.grid_mesh(80, 80, 4.0, 4.0, lambda X, Z: 0.0 * X, x0=-2.0, z0=-2.0)
    bb.parts = [dict(tri_start=0, tri_count=bb.ntris,
                     mat=scenes.default_material(backface_culling=0, billboard=1, billboard_lock=(0, 1, 0)))]
    base = scenes.feature_scene(5, n=4)
    sd = scenes.SceneData([tube, grid, bb], 3, [base.lights[i] for i in range(base.nlights)], base.lists,
                          cells=base.cells[:base.ncells], name="big_altered")
    pos = np.array([(0.0, -1.5, -8.0), (0.0, -2.0, -7.0), (3.0, 1.0, -10.0)], np.float32)
    scenes.set_models_trs(sd, [0, 1, 2], pos, np.ones((3, 3), np.float32), scenes.ident(3), frustum=0)
    sd.mv["skinned"][0] = 1
    sd.bones = scenes.tube_bones(rng, 1, pos[:1], 4, bend=0.8)
    sd.subdivision_levels = np.array([(100.0, 0.05), (400.0, 0.2)], np.float32)
    sd.max_subdivisions = 2
    cam = scenes.feature_camera("persp")
    ref = pyoracle.render(sd, cam)
    assert max(s["capacity"] for s in ref.segments) > 2 * 2048
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            assert_frames_equal(ctx.download(), ref, f"big altered/mode{mode}")
    finally:
        ctx.release(sid)


@pytest.mark.parametrize("kind", scenes.FRAME_VARIANTS)
def test_full_frame_variants_match_oracle(ctx, kind):
    """The full 4096-model frame (69.7 M triangles, 1920x1080) with one feature on for every model
    -- shape keys, skinning, billboards, auto-subdivision, dynamic batching -- bit for bit against
    the oracle (run on all host threads)."""
    import os
    sd = scenes.frame_variant(kind)
    ref = pyoracle.render(sd, sd.camera, threads=os.cpu_count() or 1)
    assert ref.visible_tris > 20_000_000
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), ref, f"frame/{kind}")
    finally:
        ctx.release(sid)


CUSTOM0_SCENES = [
    ("sphere", lambda: scenes.uv_sphere_scene(1)),
    ("cubes", lambda: scenes.small_variant("cubes", 3)),
    ("features", lambda: scenes.feature_scene(5)),
    ("skinned", lambda: scenes.skinned_scene(7)),
    ("billboards", lambda: scenes.billboard_scene(9)),
    ("subdivision", lambda: scenes.subdivision_scene(10)),
    ("batches", lambda: scenes.batch_scene(11)),
    ("nested_lights", lambda: scenes.nested_light_scene(6)),
]


@pytest.mark.parametrize("name,make", CUSTOM0_SCENES, ids=[c[0] for c in CUSTOM0_SCENES])
@pytest.mark.parametrize("variant", ["persp", "tilted", "ortho"])
def test_custom0_stream_matches_oracle(ctx, name, make, variant):
    """Perspective-corrected texture mapping: every corner's UV / w and Custom0 = 1 / w
    (camera.go:1689-1704) on the meshlet, record, skinned, billboard and subdivided routes,
    both forms, bit for bit against the oracle."""
    sd = make()
    cam = scenes.corrected_camera(variant)
    ref = pyoracle.render(sd, cam)
    assert ref.custom0 is not None and ref.visible_tris > 0
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_BATCHED, abi.MODE_PLAIN):
            ctx.render(sid, cam, mode=mode)
            got = ctx.download()
            assert_frames_equal(got, ref, f"custom0/{name}/{variant}/mode{mode}")
            c0 = ctx.download_custom0()
            assert np.array_equal(bits(c0), bits(ref.custom0)), f"custom0/{name}/{variant}/mode{mode}: Custom0"
    finally:
        ctx.release(sid)


def test_custom0_only_for_corrected_jobs(ctx):
    """Two jobs in one launch, one with perspective-corrected mapping: Custom0 holds 1 / w for
    its corners and 0 for the other job's; a frame without the option has no Custom0."""
    sd = scenes.feature_scene(5)
    sid = ctx.upload(sd)
    try:
        cams = [scenes.corrected_camera("persp"), scenes.feature_camera("tilted")]
        ctx.render_jobs([job(sid, c, None) for c in cams])
        got = ctx.download()
        c0 = ctx.download_custom0()
        parts = split_jobs(got, 2)
        for j, cam in enumerate(cams):
            assert_frames_equal(parts[j], pyoracle.render(sd, cam), f"custom0 jobs/{j}")
        b, sel = 0, [[], []]
        for s in got.segments:
            sel[s["job"]].extend(range(b, b + s["count"]))
            b += s["count"]
        assert np.array_equal(bits(c0[sel[0]]), bits(pyoracle.render(sd, cams[0]).custom0))
        assert not c0[sel[1]].any()
        ctx.render(sid, scenes.feature_camera("persp"))
        ctx.sync()
        with pytest.raises(abi.T3DError):
            ctx.download_custom0()
    finally:
        ctx.release(sid)


def test_autotune_leaves_a_bit_exact_tuning(ctx):
    """The autotuner sweeps launch shape x tile size (re-cutting the meshlets) and the vertex
    chunk, leaves the context on the fastest setting, and that setting renders the oracle's bits."""
    from tetra3d_gb300 import autotune
    sd = scenes.small_variant("batched", 21)
    sid = ctx.upload(sd)
    try:
        best, res = autotune.tune(ctx, sid, sd.camera, frames=2, tiles=(1024, 2048), splits=(1, 0), chunks=(2048, 4096))
        shapes = {k: v for k, v in res.items() if len(k) == 3}
        assert len(shapes) == 4 and best[:3] in shapes
        assert shapes[best[:3]] == min(shapes.values())
        ctx.render(sid, sd.camera)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), f"after autotune {best}")
    finally:
        ctx.set_tuning(tile_tris=2048, block_threads=256, vertex_chunk=4096)
        ctx.set_split_phases(1)
        ctx.release(sid)


def test_deferred_readback_pipelines_frames(ctx):
    """t3d_frame_readback / t3d_frame_collect: with frame i + 1 queued before frame i's counts are
    collected, every collected frame reports its own counts (those of the synchronous path)."""
    sd = scenes.feature_scene(5)
    sid = ctx.upload(sd)
    try:
        cams = [scenes.feature_camera(v) for v in ("persp", "tilted", "ortho", "persp")]
        expect = []
        for c in cams:
            ctx.render(sid, c, mode=abi.MODE_BATCHED)
            expect.append(int(ctx.sync().visible_tris))
        assert len(set(expect)) > 1  # distinct counts, so a mix-up would show
        got = []
        ctx.render(sid, cams[0], mode=abi.MODE_BATCHED)
        for k in range(len(cams)):
            ctx.readback()
            if k + 1 < len(cams):
                ctx.render(sid, cams[k + 1], mode=abi.MODE_BATCHED)
            got.append(int(ctx.collect().visible_tris))
        assert got == expect
        assert int(ctx.sync().visible_tris) == expect[-1]
        assert_frames_equal(ctx.download(), pyoracle.render(sd, cams[-1]), "after pipelined frames")
        # one read-back at a time; a collect needs a read-back
        ctx.readback()
        assert ctx.lib.t3d_frame_readback(ctx.h) == abi.T3D_E_INVAL
        ctx.collect()
        assert ctx.lib.t3d_frame_collect(ctx.h, None) == abi.T3D_E_INVAL
    finally:
        ctx.release(sid)


def test_parts_of_many_tiles_scan_in_chunks(ctx):
    """A 1024^2 terrain alone: four parts of about 256 meshlet tiles each, far more than the
    frame's tiles per block of the scan phase, so each pair's cross-tile scan runs as one work
    item per chunk of 32 tiles (the chunks' bin counts summed by the histogram phase). Every form
    and launch shape gives the oracle's stream."""
    sd = scenes.terrain_scene(5, n=1024, w=1280, h=720)
    cam = sd.camera
    ref = pyoracle.render(sd, cam, threads=os.cpu_count() or 1)
    assert ref.visible_tris > 100000
    assert max(s["capacity"] for s in ref.segments) > 128 * 2048  # parts of more than 128 full tiles
    sid = ctx.upload(sd)
    try:
        for mode, split in FORMS:
            ctx.set_split_phases(split)
            ctx.render(sid, cam, mode=mode)
            assert_frames_equal(ctx.download(), ref, f"terrain1024/mode{mode}/split{split}")
    finally:
        ctx.set_split_phases(1)
        ctx.release(sid)


def test_shape_keyed_meshlets_follow_weight_changes(ctx):
    """Shape-keyed meshes take the meshlet route, their meshlets cut from the keyed streams baked
    for the current weights: new weights refill the meshlets, a re-cut for another tile size starts
    from the current weights, and both routes at both tile sizes give the oracle's stream."""
    sd = scenes.frame_variant("shape_keys", n=128)
    cam = sd.camera
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, cam, threads=os.cpu_count() or 1), "initial")
        for step, w in enumerate(([0.1, 0.9], [-0.7, 0.25])):
            for m in (0, len(sd.meshes) - 1):
                sd.meshes[m].shape_weights = np.array(w, np.float32)
                ctx.set_shape_weights(sid, m, sd.meshes[m].shape_weights)
            ref = pyoracle.render(sd, cam, threads=os.cpu_count() or 1)
            for tile in (2048, 1024):
                ctx.set_tuning(tile_tris=tile)
                for meshlets in (1, 0):
                    ctx.set_meshlets(meshlets)
                    ctx.render(sid, cam)
                    assert_frames_equal(ctx.download(), ref, f"weights{step}/tile{tile}/meshlets{meshlets}")
    finally:
        ctx.set_meshlets(1)
        ctx.set_tuning(tile_tris=2048)
        ctx.release(sid)
