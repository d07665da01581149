"""t3d_frame_raster (the colour and depth passes of flush on the device) against its oracle,
bit for bit, on the emitted stream of real frames: opaque and transparent pairs, depth rendering
on and off, fog in the colour pass with every curve and with dithering, several jobs."""
import numpy as np
import pytest

from tetra3d_gb300 import abi, scenes
from tetra3d_gb300.runtime import job
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _fog_depth_camera(variant):
    """Depth rendering on with World fog: the colour pass applies the fog (base3d.kage)."""
    c = scenes.feature_camera("persp")
    c.fog_on, c.fog_mode = 1, {"add": abi.FOG_ADD, "sub": abi.FOG_SUB, "over": abi.FOG_OVERWRITE}[variant]
    c.fog_range[:] = [0.2, 0.9]
    c.fog_color[:] = [0.3, 0.5, 0.9, 1.0]
    return c


CASES = [
    ("sphere", lambda: (scenes.uv_sphere_scene(1), None), {}),
    ("cubes", lambda: (scenes.small_variant("cubes", 3), None), {}),
    ("terrain", lambda: (scenes.small_variant("terrain", 3), None), {}),
    ("features_persp", lambda: (scenes.feature_scene(5), scenes.feature_camera("persp")), {}),
    ("features_tilted", lambda: (scenes.feature_scene(6), scenes.feature_camera("tilted")), {}),
    ("features_no_depth_fog", lambda: (scenes.feature_scene(5), scenes.feature_camera("fog_add")), {}),
    ("features_ortho", lambda: (scenes.feature_scene(7), scenes.feature_camera("ortho")), {}),
    ("fog_add_linear", lambda: (scenes.feature_scene(5), _fog_depth_camera("add")), {}),
    ("fog_sub_outcirc", lambda: (scenes.feature_scene(6), _fog_depth_camera("sub")), {"fog_curve": 1}),
    ("fog_over_incirc_dither", lambda: (scenes.feature_scene(7), _fog_depth_camera("over")),
     {"fog_curve": 2, "dither_size": 2.0}),
    ("fogless", lambda: (scenes.feature_scene(5), _fog_depth_camera("add")), {"fogless": 1}),
    # dynamic batches: the members of a batch share one depth composite
    ("batches", lambda: (scenes.batch_scene(11), scenes.feature_camera("persp")), {}),
    ("batches_tilted_fog", lambda: (scenes.batch_scene(12), _fog_depth_camera("add")), {}),
]


@pytest.mark.parametrize("name,make,opts", CASES, ids=[c[0] for c in CASES])
def test_raster_matches_oracle(ctx, name, make, opts):
    sd, cam = make()
    cam = cam if cam is not None else sd.camera
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam)
        col, dep = ctx.raster(**opts)
    finally:
        ctx.release(sid)
    f = pyoracle.render(sd, cam)
    ocol, odep = pyoracle.raster(f, sd, cam, **opts)
    assert (ocol[..., 3] > 0).sum() > 100, "the scene covers pixels"
    bad = np.argwhere(np.any(col != ocol, axis=-1))
    assert bad.size == 0, f"{name}: colour differs at {len(bad)} pixels, first {bad[:3].tolist()}: " \
                          f"gpu {col[tuple(bad[0])]} oracle {ocol[tuple(bad[0])]}"
    assert np.array_equal(dep, odep), f"{name}: depth image differs"


def test_raster_second_job(ctx):
    a, b = scenes.feature_scene(5), scenes.uv_sphere_scene(2)
    sa, sb = ctx.upload(a), ctx.upload(b)
    try:
        cam_b = b.camera
        ctx.render_jobs([job(sa, scenes.feature_camera("persp")), job(sb, cam_b)])
        col, dep = ctx.raster(job=1)
    finally:
        ctx.release(sa)
        ctx.release(sb)
    ocol, odep = pyoracle.raster(pyoracle.render(b, cam_b), b, cam_b)
    assert np.array_equal(col, ocol) and np.array_equal(dep, odep)


# ---- textures and alpha clip: base3d.kage's filters and mappings, the clip-alpha shader ----

def _tiled_uvs(sd, lo=-1.0, hi=2.0):
    """Mesh UVs spread over [lo, hi]: negative and past-the-edge texture coordinates that the
    samplers wrap (mod in the colour pass, fract in the clip-alpha pass)."""
    for m in sd.meshes:
        m.uvs = np.ascontiguousarray(m.uvs * np.float32(hi - lo) + np.float32(lo), np.float32)
    return sd


TEX_CASES = [
    ("textured_persp", lambda: (scenes.textured_scene(21), scenes.feature_camera("persp")), {}),
    ("textured_tilted", lambda: (scenes.textured_scene(22), scenes.feature_camera("tilted")), {}),
    ("textured_fog_outcirc", lambda: (scenes.textured_scene(23), _fog_depth_camera("add")), {"fog_curve": 1}),
    ("textured_ortho", lambda: (scenes.textured_scene(24), scenes.feature_camera("ortho")), {}),
    ("textured_no_depth", lambda: (scenes.textured_scene(25), scenes.feature_camera("fog_add")), {}),
    ("textured_batches", lambda: (scenes.texture_materials(scenes.batch_scene(12), 12), scenes.feature_camera("persp")),
     {}),
    ("textured_tiled_uvs", lambda: (_tiled_uvs(scenes.textured_scene(26)), scenes.feature_camera("tilted")), {}),
    # perspective-corrected texture mapping: UV / w and Custom0 = 1 / w interpolated, divided per pixel
    ("textured_corrected", lambda: (scenes.textured_scene(27), scenes.feature_camera("corrected")), {}),
    ("textured_corrected_tilted", lambda: (scenes.textured_scene(28), scenes.corrected_camera("tilted")), {}),
    ("textured_corrected_ortho", lambda: (scenes.textured_scene(29), scenes.corrected_camera("ortho")), {}),
    ("textured_corrected_no_depth", lambda: (scenes.textured_scene(30), scenes.corrected_camera("fog_add")), {}),
    ("textured_corrected_tiled_uvs", lambda: (_tiled_uvs(scenes.textured_scene(31)), scenes.feature_camera("corrected")),
     {}),
]


@pytest.mark.parametrize("name,make,opts", TEX_CASES, ids=[c[0] for c in TEX_CASES])
def test_textured_raster_matches_oracle(ctx, name, make, opts):
    sd, cam = make()
    tex = scenes.raster_textures(seed=len(name))
    ctx.set_textures(tex)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam)
        col, dep = ctx.raster(**opts)
    finally:
        ctx.release(sid)
        ctx.set_textures([])
    f = pyoracle.render(sd, cam)
    ocol, odep = pyoracle.raster(f, sd, cam, textures=tex, **opts)
    plain, _ = pyoracle.raster(f, sd, cam, **opts)
    assert (ocol[..., 3] > 0).sum() > 100, "the scene covers pixels"
    assert np.any(ocol != plain), "the textures change the image"
    bad = np.argwhere(np.any(col != ocol, axis=-1))
    assert bad.size == 0, f"{name}: colour differs at {len(bad)} pixels, first {bad[:3].tolist()}: " \
                          f"gpu {col[tuple(bad[0])]} oracle {ocol[tuple(bad[0])]}"
    assert np.array_equal(dep, odep), f"{name}: depth image differs"


def test_texture_errors(ctx):
    sd = scenes.textured_scene(21)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, scenes.feature_camera("persp"))
        ctx.set_textures(scenes.raster_textures()[:1])   # materials name textures 2 and 3 too
        with pytest.raises(abi.T3DError):
            ctx.raster()
        ctx.set_textures(scenes.raster_textures())
        ctx.render(sid, scenes.feature_camera("persp"))
        col, _ = ctx.raster()
        assert col[..., 3].any()
    finally:
        ctx.release(sid)
        ctx.set_textures([])
    with pytest.raises(abi.T3DError):
        ctx.set_textures([np.zeros((0, 4, 4), np.uint8)])


@pytest.mark.parametrize("shared", [-1, 7, 0])
def test_large_triangles_shared_or_per_warp(ctx, shared):
    """Triangles with a pixel box over 32 pixels are shared out to the grid in 1024-pixel chunks
    up to the list's capacity, and rasterised by their own warp past it (-1: none shared, 7: the
    first seven): the images are the oracle's either way. The scene has thousands of such
    triangles, hundreds over one chunk."""
    sd, cam = scenes.textured_scene(21), scenes.feature_camera("tilted")
    tex = scenes.raster_textures(seed=3)
    ctx.set_textures(tex)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, cam)
        col, dep = ctx.raster(shared_large_tris=shared)
    finally:
        ctx.release(sid)
        ctx.set_textures([])
    ocol, odep = pyoracle.raster(pyoracle.render(sd, cam), sd, cam, textures=tex)
    assert np.array_equal(col, ocol) and np.array_equal(dep, odep)


def test_raster_edge_cases(ctx):
    """Nothing visible (the camera looks away): both images stay cleared. Images of 1x1, 3x2
    and 7x5 pixels (fewer pixels than a block or a warp) and a 3x3 orthographic view against
    the oracle. A job with no render pair (an empty scene) rasterises to cleared images."""
    sd = scenes.uv_sphere_scene(1)
    sid = ctx.upload(sd)
    try:
        away = scenes.camera(w=64, h=48, rot=scenes.rotate(0, 1, 0, float(np.pi)), fov=75.0)
        ctx.render(sid, away)
        assert ctx.sync().visible_tris == 0
        col, dep = ctx.raster()
        assert col.shape == (48, 64, 4) and not col.any() and not dep.any()
        near = (0.0, 0.0, -3.0)  # two units from the sphere's centre: it fills the small views
        cams = [scenes.camera(pos=near, w=w, h=h, fov=75.0) for w, h in ((1, 1), (3, 2), (7, 5))]
        cams.append(scenes.camera(pos=near, w=3, h=3, perspective=0, ortho_scale=3.0))
        for cam in cams:
            ctx.render(sid, cam)
            col, dep = ctx.raster()
            ocol, odep = pyoracle.raster(pyoracle.render(sd, cam), sd, cam)
            assert col.shape == (cam.height, cam.width, 4)
            assert np.array_equal(col, ocol) and np.array_equal(dep, odep), (cam.width, cam.height)
            assert ocol[..., 3].any(), "the sphere covers pixels"
    finally:
        ctx.release(sid)
    empty = scenes.SceneData([scenes.quad_mesh(1.0, 1.0)], 0, [], [[]], name="empty")
    eid = ctx.upload(empty)
    try:
        ctx.render(eid, scenes.camera(w=16, h=16))
        col, dep = ctx.raster()
        assert not col.any() and not dep.any()
    finally:
        ctx.release(eid)


def test_raster_full_frame_textured_matches_oracle(ctx):
    """The full 4096-model frame (26 M visible triangles at 1920x1080) with textured materials
    (three textures, both filters, UV and screen mapping, alpha clip on some), rasterised on the
    device and by the raster oracle from the downloaded stream (the stream itself is checked
    against the vertex-stage oracle elsewhere)."""
    sd = scenes.texture_materials(scenes.batched_scene(4, n=4096), 7)
    tex = scenes.raster_textures()
    ctx.set_textures(tex)
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera)
        fr = ctx.download()
        col, dep = ctx.raster()
    finally:
        ctx.release(sid)
        ctx.set_textures([])
    assert fr.visible_tris > 20_000_000
    ocol, odep = pyoracle.raster(fr, sd, sd.camera, textures=tex)
    bad = np.argwhere(np.any(col != ocol, axis=-1))
    assert bad.size == 0, f"colour differs at {len(bad)} pixels, first {bad[:3].tolist()}"
    assert np.array_equal(dep, odep)
