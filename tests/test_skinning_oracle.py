"""The oracle's shape keys and skinning (Mesh.VertexPositionWithShapeKeys,
Model.skinVertex) against equivalences that hold value for value:

- identity bones with weight 1, with two half weights on the same bone, and with a
  1.0 weight after a partial one on a different bone (skinVertex stops at the 1.0)
  give the unskinned model under an identity transform;
- shape keys give the same corners as a mesh whose base positions and normals
  hold the keyed values (the depth keys differ: tri.Center stays on the base
  positions, so triangles are matched by index, not by draw order);
- a skinned model behind the camera is culled on its own position.
"""
import numpy as np

from oracle import pyoracle
from tetra3d_gb300 import scenes

F32 = np.float32


def _one_model_scene(mesh, skinned, bones=None, nlights=True):
    base = scenes.feature_scene(5, n=4)
    lights = [base.lights[i] for i in range(base.nlights)] if nlights else []
    sd = scenes.SceneData([mesh], 1, lights, base.lists if nlights else [[]],
                          cells=base.cells[:base.ncells] if nlights else None, name="one")
    scenes.set_models_trs(sd, [0], np.zeros((1, 3), F32), np.ones((1, 3), F32), scenes.ident(1), frustum=0)
    sd.mv["skinned"][0] = int(skinned)
    sd.bones = bones
    cam = scenes.camera(pos=(0.0, 1.0, 6.0), w=640, h=360, fov=60.0, near=0.1, far=60.0)
    sd.camera = cam
    return sd, cam


def _tube(rng):
    t = scenes.tube_mesh(rings=6, segments=8)
    t.parts = [dict(tri_start=0, tri_count=t.ntris // 2, mat=scenes.default_material(lighting_mode=0)),
               dict(tri_start=t.ntris // 2, tri_count=t.ntris - t.ntris // 2,
                    mat=scenes.default_material(lv_shading_mode=2, backface_culling=0))]
    t.colors = rng.uniform(0.4, 1.0, (t.nverts, 4)).astype(F32)
    return t


def _value_equal(a, b, what):
    assert [(s["model"], s["part"], s["count"]) for s in a.segments] == \
           [(s["model"], s["part"], s["count"]) for s in b.segments], what
    assert np.array_equal(a.tri_index, b.tri_index), what
    for name in ("xyuv", "rgba", "depth"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), f"{what}: {name}"


def test_identity_bones_equal_unskinned():
    rng = np.random.default_rng(3)
    t = _tube(rng)
    V = t.nverts
    bones = np.stack([scenes.ident(), scenes.ident() * F32(7.5), scenes.ident()]).astype(F32)
    bones[1][3, :3] = (3.0, -2.0, 1.0)  # a bone that must never contribute
    plain, cam = _one_model_scene(t, skinned=False)
    ref = pyoracle.render(plain, cam)
    assert ref.visible_tris > 20
    for kind in ("one", "halves", "stop"):
        j = np.zeros((V, 4), np.uint32)
        w = np.zeros((V, 4), F32)
        if kind == "one":
            j[:, 0], w[:, 0] = 0, 1.0
        elif kind == "halves":
            j[:, :2], w[:, :2] = 2, 0.5
        else:  # partial weight on the odd bone, then 1.0 on the identity: skinVertex keeps the identity
            j[:, 0], w[:, 0] = 1, 0.25
            j[:, 1], w[:, 1] = 0, 1.0
            j[:, 2], w[:, 2] = 1, 0.5
        t.joints, t.weights = j, w
        sk, _ = _one_model_scene(t, skinned=True, bones=bones)
        _value_equal(pyoracle.render(sk, cam), ref, kind)
    # the odd bone does change the result when it is reached
    j = np.zeros((V, 4), np.uint32)
    w = np.zeros((V, 4), F32)
    j[:, 0], w[:, 0] = 1, 0.25
    j[:, 1], w[:, 1] = 0, 0.75
    t.joints, t.weights = j, w
    sk, _ = _one_model_scene(t, skinned=True, bones=bones)
    got = pyoracle.render(sk, cam)
    assert got.visible_tris != ref.visible_tris or not np.array_equal(got.xyuv, ref.xyuv)


def _by_triangle(frame):
    out = {}
    b = 0
    for s in frame.segments:
        for k in range(s["count"]):
            out[(s["part"], int(frame.tri_index[b + k]))] = (frame.xyuv[b + k], frame.rgba[b + k])
        b += s["count"]
    return out


def test_shape_keys_equal_baked_mesh():
    rng = np.random.default_rng(4)
    sph = scenes.uv_sphere(12, 6, 1.0)
    sph.parts = [dict(tri_start=0, tri_count=sph.ntris, mat=scenes.default_material(backface_culling=0))]
    K = 3
    dp = rng.uniform(-0.3, 0.3, (K, sph.nverts, 3)).astype(F32)
    dn = rng.uniform(-0.3, 0.3, (K, sph.nverts, 3)).astype(F32)
    wk = np.array([0.5, -0.75, 0.3], F32)
    sph.shape_positions, sph.shape_normals, sph.shape_weights = dp, dn, wk
    keyed, cam = _one_model_scene(sph, skinned=False)
    got = pyoracle.render(keyed, cam)
    pos, nrm = sph.positions.copy(), sph.normals.copy()
    for k in range(K):  # out += delta * weight, key by key, in float32
        pos = (pos + dp[k] * wk[k]).astype(F32)
        nrm = (nrm + dn[k] * wk[k]).astype(F32)
    baked = scenes.MeshData(pos, nrm, sph.uvs, sph.indices, parts=sph.parts, dims=None)
    # tri.Center and Dimensions stay on the base mesh in the reference
    baked.dims = (sph.positions.min(0), sph.positions.max(0))
    plain, _ = _one_model_scene(baked, skinned=False)
    ref = pyoracle.render(plain, cam)
    a, b = _by_triangle(got), _by_triangle(ref)
    assert len(a) > 20 and set(a) == set(b)
    for key in a:
        assert np.array_equal(a[key][0], b[key][0]) and np.array_equal(a[key][1], b[key][1]), key
    # zero weights leave the mesh as it is
    sph.shape_weights = np.zeros(K, F32)
    zero, _ = _one_model_scene(sph, skinned=False)
    sph2 = scenes.MeshData(sph.positions, sph.normals, sph.uvs, sph.indices, parts=sph.parts)
    none, _ = _one_model_scene(sph2, skinned=False)
    _value_equal(pyoracle.render(zero, cam), pyoracle.render(none, cam), "zero weights")


def test_skinned_scene_draws_and_culls():
    sd = scenes.skinned_scene(7)
    for v in ("persp", "ortho", "tilted"):
        r = pyoracle.render(sd, scenes.feature_camera(v))
        drawn = {s["model"] for s in r.segments if s["count"]}
        assert any(sd.mv["skinned"][m] for m in drawn) and any(not sd.mv["skinned"][m] for m in drawn)
        assert not any(s["count"] for s in r.segments if s["model"] == 1)  # behind the camera
        assert r.culled_models >= 1
