"""The oracle's auto-subdivision (Mesh.SetAutoSubdivide, Triangle.handleSubdivision)
against known answers: one large triangle seen from near draws the level whose
MaximumTriangleSize its MaxSpan halves down to (4, 16 or 64 triangles), the
subdivision count clamps the level, a far camera draws the base triangles exactly
as the unsubdivided mesh does, and the subdivided corners interpolate the base
triangle's corners."""
import numpy as np
import pytest

from oracle import pyoracle
from tetra3d_gb300 import scenes

F32 = np.float32


def _triangle_scene(levels, max_sub, auto=1, z=-4.0):
    # MaxSpan 8: the edge from (-4, -2) to (4, -2)
    pos = np.array([(-4.0, -2.0, 0.0), (4.0, -2.0, 0.0), (0.0, 3.0, 0.0)], F32)
    nrm = np.tile(np.array([0, 0, 1], F32), (3, 1))
    uv = np.array([(0, 0), (1, 0), (0.5, 1)], F32)
    me = scenes.MeshData(pos, nrm, uv, np.array([(0, 1, 2)], np.uint32))
    me.colors = np.array([(1, 0, 0, 1), (0, 1, 0, 1), (0, 0, 1, 1)], F32)
    me.parts = [dict(tri_start=0, tri_count=1, mat=scenes.default_material(backface_culling=0, shadeless=1))]
    me.auto_subdivide = auto
    sd = scenes.SceneData([me], 1, [], [[]], name="tri")
    scenes.set_models_trs(sd, [0], np.array([(0.0, 0.0, z)], F32), np.ones((1, 3), F32), scenes.ident(1), frustum=0)
    sd.subdivision_levels = np.array(levels, F32)
    sd.max_subdivisions = max_sub
    cam = scenes.camera(w=640, h=480, fov=90.0, near=0.05, far=100.0)
    cam.fog_on = 0
    return sd, cam


@pytest.mark.parametrize("size,max_sub,want", [(1.0, 3, 64), (2.0, 3, 16), (5.0, 3, 4), (9.0, 3, 1),
                                               (1.0, 1, 4), (1.0, 2, 16)])
def test_level_choice_near(size, max_sub, want):
    sd, cam = _triangle_scene([(100.0, size)], max_sub)
    r = pyoracle.render(sd, cam)
    assert r.visible_tris == want


def test_far_camera_draws_the_base():
    sd, cam = _triangle_scene([(4.0, 1.0)], 3, z=-30.0)  # farther than DistanceSquared 4
    plain, _ = _triangle_scene([(4.0, 1.0)], 3, auto=0, z=-30.0)
    a, b = pyoracle.render(sd, cam), pyoracle.render(plain, cam)
    assert a.visible_tris == b.visible_tris == 1
    for name in ("xyuv", "rgba", "depth"):
        assert np.array_equal(getattr(a, name), getattr(b, name))


def test_closest_level_wins():
    # both levels contain the camera distance; the one with the smaller DistanceSquared applies
    sd, cam = _triangle_scene([(400.0, 5.0), (100.0, 1.0)], 3)
    assert pyoracle.render(sd, cam).visible_tris == 64
    sd, cam = _triangle_scene([(100.0, 5.0), (400.0, 1.0)], 3)
    assert pyoracle.render(sd, cam).visible_tris == 4


def test_subdivided_corners_interpolate():
    """Level 0 of the triangle: the four children's UVs are the corners' and edge midpoints' UVs."""
    sd, cam = _triangle_scene([(100.0, 5.0)], 3)
    cam.perspective_corrected = 0
    me = sd.meshes[0]
    me.parts[0]["mat"]["tex_w"], me.parts[0]["mat"]["tex_h"] = 1.0, 1.0
    r = pyoracle.render(sd, cam)
    assert r.visible_tris == 4
    uv = np.round(r.xyuv[:, :, 2:4].reshape(-1, 2), 6)
    got = {tuple(x) for x in uv}
    corners = [(0.0, 1.0), (1.0, 1.0), (0.5, 0.0)]  # (u, 1 - v)
    mids = [(0.5, 1.0), (0.75, 0.5), (0.25, 0.5)]
    assert got == set(corners) | set(mids)


def test_subdivision_scene_draws_levels():
    sd = scenes.subdivision_scene(10)
    r = pyoracle.render(sd, scenes.feature_camera("persp"))
    plain_caps = {int(m): sd.meshes[int(m)].ntris for m in sd.mv["mesh"]}
    # some subdivided part draws more triangles than its mesh has
    counts = {}
    for s in r.segments:
        m = int(sd.mv["mesh"][s["model"]])
        if sd.meshes[m].auto_subdivide:
            counts[s["model"]] = counts.get(s["model"], 0) + s["count"]
    assert any(c > plain_caps[int(sd.mv["mesh"][k])] for k, c in counts.items())


def test_timing_renderer_counts_like_render():
    """pyoracle.Renderer, the CPU arms' timing path (output arrays allocated once and reused),
    counts the visible triangles render() does, also for auto-subdivided meshes, which list more
    triangles than the scene holds (its arrays grow once), and on repeated calls."""
    from tetra3d_gb300 import scenes
    for sd, cam in ((scenes.uv_sphere_scene(1), None), (scenes.subdivision_scene(10), scenes.feature_camera("persp"))):
        cam = cam or sd.camera
        r = pyoracle.Renderer(sd, cam)
        want = pyoracle.render(sd, cam).visible_tris
        assert want > 0
        assert r.render() == want
        assert r.render(threads=2) == want
