"""Host logic on the CPU (oracle and scene generators, no GPU): draw order of render pairs,
independence of render pairs (what makes replicas and model subsets valid), light masks,
animation steps, light-volume cell counts, and the workload generators' sizes."""
import numpy as np
import pytest

from tetra3d_gb300 import abi, scenes
from oracle import pyoracle

F = np.float32


def _is_transparent(md, mat):
    """Model.isTransparent / MeshPart transparency (model.go:1086-1107, material.go:192-207)."""
    if mat["present"]:
        mat_t = (mat["transparency_mode"] == abi.TRANSPARENCY_TRANSPARENT or not mat["blend_source_over"]
                 or (mat["transparency_mode"] == abi.TRANSPARENCY_AUTO and F(mat["color"][3]) < F(0.999)))
        model_t = mat["transparency_mode"] != abi.TRANSPARENCY_OPAQUE and F(md["color"][3]) < F(0.999)
        return bool(mat_t or model_t)
    return bool(F(md["color"][3]) < F(0.999))


def _slices(frame):
    """(model, part) -> (xyuv, rgba, depth) of that render pair (the frame is compacted in draw order)."""
    out, b = {}, 0
    for s in frame.segments:
        n = s["count"]
        out[(s["model"], s["part"])] = (frame.xyuv[b:b + n], frame.rgba[b:b + n], frame.depth[b:b + n])
        b += n
    return out


def _bits_equal(a, b):
    return all(np.array_equal(np.asarray(x, F).view(np.uint32), np.asarray(y, F).view(np.uint32)) for x, y in zip(a, b))


@pytest.mark.parametrize("variant", ["persp", "fog_add"])
def test_draw_order_solids_then_transparents(variant):
    sd = scenes.feature_scene(5)
    cam = scenes.feature_camera(variant)
    f = pyoracle.render(sd, cam)
    campos = np.array(cam.transform, F).reshape(4, 4)[3, :3]
    kinds, keys = [], []
    for s in f.segments:
        md = sd.mv[s["model"]]
        mat = sd.meshes[int(md["mesh"])].parts[s["part"]]["mat"]
        kinds.append(_is_transparent(md, mat))
        d = campos - sd.mv["transform"][s["model"]].reshape(4, 4)[3, :3]
        keys.append((mat["render_order"] if mat["present"] else 0, -float(((d[0] * d[0]) + d[1] * d[1]) + d[2] * d[2])))
    assert any(kinds) and not all(kinds)
    first_t = kinds.index(True)
    assert all(kinds[first_t:]), "every solid pair precedes every transparent one"
    # transparents: render order ascending, then far to near (camera.go:2050-2055)
    tk = keys[first_t:]
    assert tk == sorted(tk)
    solids = f.segments[:first_t]
    if cam.render_depth:  # solids keep the model list order (camera.go:1343-1457)
        order = [(s["model"], s["part"]) for s in solids]
        assert order == sorted(order)
    else:  # depth off: solids are sorted like transparents (camera.go:1461-1470)
        assert keys[:first_t] == sorted(keys[:first_t])


def test_render_pairs_are_independent():
    """A render pair's triangles depend only on its model, part, lights and camera: rendering a subset
    of the models gives the same bits for every pair it keeps."""
    sd = scenes.feature_scene(7)
    cam = scenes.feature_camera("tilted")
    full = _slices(pyoracle.render(sd, cam))
    keep = np.arange(0, sd.nmodels, 3)
    sub = scenes.subset(sd, keep)
    part = _slices(pyoracle.render(sub, cam))
    assert part
    for (m, p), v in part.items():
        assert _bits_equal(v, full[(int(keep[m]), p)]), (m, p)


def test_light_mask_equals_dropping_the_light():
    sd = scenes.small_variant("batched", 3)
    drop = 2
    mask = ((1 << 128) - 1) & ~(1 << drop)
    masked = pyoracle.render(sd, sd.camera, light_mask=mask)
    sd2 = scenes.small_variant("batched", 3)
    sd2.lists = [[x for x in lst if x != drop] for lst in sd2.lists]
    dropped = pyoracle.render(sd2, sd2.camera)
    assert masked.segments == dropped.segments
    assert _bits_equal((masked.xyuv, masked.rgba, masked.depth), (dropped.xyuv, dropped.rgba, dropped.depth))
    full = pyoracle.render(sd, sd.camera)
    assert not np.array_equal(full.rgba, masked.rgba)


def test_animation_frames_equal_host_rotations():
    """animate_frames=k applies Node.Rotate k times in the frame (rot = step * rot, matrix.go:583-585);
    the same rotations composed on the host give the same frame."""
    sd = scenes.small_variant("batched", 5)
    k = 3
    anim = pyoracle.render(sd, sd.camera, animate_frames=k)
    n = sd.nmodels
    rot = sd.mv["rotation"].reshape(n, 4, 4).copy()
    step = sd.mv["rotate_step"].reshape(n, 4, 4)
    for _ in range(k):
        rot = scenes.mult(step, rot)
    sd.mv["rotation"] = rot.reshape(n, 16)
    host = pyoracle.render(sd, sd.camera)
    assert anim.segments == host.segments
    assert _bits_equal((anim.xyuv, anim.rgba, anim.depth), (host.xyuv, host.rgba, host.depth))


def test_culled_and_skipped_models():
    sd = scenes.feature_scene(5)
    f = pyoracle.render(sd, sd.camera)
    counts = {}
    for s in f.segments:
        counts.setdefault(s["model"], 0)
        counts[s["model"]] += s["count"]
    assert counts.get(0, 0) == 0, "model behind the camera draws nothing"
    assert counts.get(1, 0) == 0, "model beyond the far plane draws nothing (frustum culling off)"
    for s in f.segments:  # an alpha-0 model draws nothing of its transparent parts (model.go:604-606)
        if s["model"] == 3 and _is_transparent(sd.mv[3], sd.meshes[int(sd.mv["mesh"][3])].parts[s["part"]]["mat"]):
            assert s["count"] == 0
    for i in np.nonzero(sd.mv["visible"] == 0)[0]:
        assert int(i) not in counts
    assert f.culled_models >= 1


def test_light_volume_counts():
    """LightVolumeResize (light.go:485-513): cells whose centres fit inside the box."""
    assert scenes.light_volume_counts([-9, -9, -9], [9, 9, 9], [4.5, 6.0, 3.0]) == [4, 3, 6]
    assert scenes.light_volume_counts([0, 0, 0], [1, 1, 1], [2, 2, 2]) == [0, 0, 0]


def test_workload_sizes():
    sd = scenes.batched_scene(4)
    assert sd.nmodels == 4096 and sd.nlights == 33
    assert (sd.total_verts(), sd.total_tris()) == (35129236, 69724700)
    assert len(sd.lists) == 4097
    t = scenes.terrain_scene(3)
    assert t.nmodels == 4 and sum(m.nverts for m in t.meshes) == 1025 * 1025  # quadrants share their seams
    c = scenes.cubes_scene(2)
    assert c.nmodels == 1000 and c.total_tris() == 12000
    s = scenes.uv_sphere_scene(1)
    assert s.total_verts() == 17 * 32


def _scene_list_scene(nlights, seed=21):
    sd = scenes.batched_scene(seed, n=24, vmin=24, vmax=1500, nlights=nlights, box=40.0, max_levels=3)
    sd.mv["light_list"] = -1  # every model lit by the scene list (list 0)
    return sd


@pytest.mark.parametrize("nlights,keep", [(8, 4), (40, 25), (40, 1)])
def test_max_light_count_keeps_the_nearest_scene_lights(nlights, keep):
    """Camera.MaxLightCount (camera.go:1474-1497): ambient first, then lights by squared distance
    from the camera; 40 lights run Go's stable sort past its 20-element insertion blocks."""
    sd = _scene_list_scene(nlights)
    cam = sd.camera
    cam.max_light_count = keep
    culled = pyoracle.render(sd, cam)
    campos = np.array(cam.transform, F).reshape(4, 4)[3, :3]
    lights = [sd.lights[i] for i in sd.lists[0]]
    def d2(L):
        p = np.array(L.transform, F).reshape(4, 4)[3, :3]
        d = campos - p
        return F(F(d[0] * d[0]) + F(d[1] * d[1])) + F(d[2] * d[2])
    order = sorted(sd.lists[0], key=lambda i: (0, 0.0) if sd.lights[i].type == abi.LIGHT_AMBIENT else (1, float(d2(sd.lights[i]))))
    explicit = _scene_list_scene(nlights)
    explicit.lists[0] = order[:keep]
    ref = pyoracle.render(explicit, explicit.camera)
    assert culled.segments == ref.segments
    assert np.array_equal(culled.rgba.view(np.uint32), ref.rgba.view(np.uint32))
    full = pyoracle.render(_scene_list_scene(nlights), _scene_list_scene(nlights).camera)
    assert not np.array_equal(full.rgba, culled.rgba)


def test_max_light_count_focus_point_and_groups():
    sd = _scene_list_scene(12)
    cam = sd.camera
    cam.max_light_count = 3
    cam.focus_set = 1
    cam.focus[:] = [30.0, 0.0, 0.0]
    a = pyoracle.render(sd, cam)
    cam.focus[:] = [-30.0, 0.0, 0.0]
    b = pyoracle.render(sd, cam)
    assert not np.array_equal(a.rgba, b.rgba)
    g = scenes.small_variant("batched", 3)  # every model in a LightGroup: MaxLightCount does not apply
    base = pyoracle.render(g, g.camera)
    g.camera.max_light_count = 1
    assert np.array_equal(pyoracle.render(g, g.camera).rgba.view(np.uint32), base.rgba.view(np.uint32))
