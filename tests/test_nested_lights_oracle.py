"""LightVolumeCell.useLights in the oracle (light.go:646-656): a vertex in a cell
gets the cell's lights (in their VertexLight form, without the model-level range
skip) added before the volume's own cell colour; in per-object mode and outside
the volume they do not apply."""
import numpy as np

from oracle import pyoracle
from tetra3d_gb300 import abi, scenes

F32 = np.float32


def _scene(lv_mode, cell_uses, pos=(0.0, 0.0, -5.0)):
    q = scenes.quad_mesh(1.0, 1.0)
    q.parts = [dict(tri_start=0, tri_count=2, mat=scenes.default_material(backface_culling=0, lv_shading_mode=lv_mode))]
    vmin, vmax, cs = np.array([-4, -4, -9], F32), np.array([4, 4, -1], F32), np.array([8, 8, 8], F32)
    counts = scenes.light_volume_counts(vmin, vmax, cs)
    assert counts == [1, 1, 1]
    amb = scenes.light(abi.LIGHT_AMBIENT, color=(0.2, 0.4, 0.6), energy=0.5)
    vol = scenes.light(abi.LIGHT_VOLUME, color=(1.0, 0.5, 0.25), energy=0.75, vol=(vmin, vmax, cs, counts, 0))
    sd = scenes.SceneData([q], 1, [vol, amb], [[0]], cells=np.array([[0.5, 0.25, 1.0, 1.0]], F32), name="nested")
    scenes.set_models_trs(sd, [0], np.array([pos], F32), np.ones((1, 3), F32), scenes.ident(1), frustum=0)
    sd.cell_uses = cell_uses
    cam = scenes.camera(w=320, h=240)
    cam.fog_on = 0
    return sd, cam


def test_cell_light_added_before_the_cell_colour():
    sd, cam = _scene(abi.LV_PER_VERTEX, [[1]])
    r = pyoracle.render(sd, cam)
    assert r.visible_tris == 2
    amb = F32(0.2) * F32(0.5), F32(0.4) * F32(0.5), F32(0.6) * F32(0.5)
    cell = (F32(0.5), F32(0.25), F32(1.0))
    col = (F32(1.0), F32(0.5), F32(0.25))
    want = [F32(F32(0) + amb[k]) + F32(F32(col[k] * cell[k]) * F32(0.75)) for k in range(3)]
    assert np.array_equal(r.rgba[:, :, :3], np.broadcast_to(np.array(want, F32), r.rgba[:, :, :3].shape))
    # without the use list: the cell colour alone
    sd2, _ = _scene(abi.LV_PER_VERTEX, [[]])
    r2 = pyoracle.render(sd2, cam)
    want2 = [F32(F32(col[k] * cell[k]) * F32(0.75)) for k in range(3)]
    assert np.allclose(r2.rgba[:, :, :3], np.array(want2, F32))


def test_cell_lights_not_in_per_object_mode_or_outside():
    sd, cam = _scene(abi.LV_PER_OBJECT, [[1]])
    plain, _ = _scene(abi.LV_PER_OBJECT, [[]])
    assert np.array_equal(pyoracle.render(sd, cam).rgba, pyoracle.render(plain, cam).rgba)
    out, _ = _scene(abi.LV_PER_VERTEX, [[1]], pos=(0.0, 0.0, -20.0))  # beyond the volume
    r = pyoracle.render(out, cam)
    assert r.visible_tris == 2 and np.all(r.rgba[:, :, :3] == 0)


def test_nested_scene_differs_from_plain():
    a = pyoracle.render(scenes.nested_light_scene(5), scenes.feature_camera("persp"))
    b = pyoracle.render(scenes.feature_scene(5), scenes.feature_camera("persp"))
    assert a.visible_tris == b.visible_tris
    assert np.array_equal(a.xyuv, b.xyuv)
    assert (a.rgba != b.rgba).any(axis=(1, 2)).sum() > 10
