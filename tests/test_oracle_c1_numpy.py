"""The C++ oracle against a second, independent restatement of the whole vertex stage
(tests/golden/make_c1_whole_path.py: numpy binary32, written directly from model.go:600-995,
light.go:110-360 and :459-724, sortingTriangles.go:38-125 and camera.go:1646-1820), on the
one-sphere scene (960 triangles, ambient + directional + point light), on the same sphere
rotated with a non-uniform scale and five lights, on that scene with a light volume in each
of its three shading modes, with the world's fog added or multiplied in, with fixed-normal and
double-sided lighting, without backface culling, front-to-back and unsorted, lit by a
LightGroup, and (oracle only) seen with perspective-corrected texture mapping (Custom0
included), vertex snapping, lighting off or an orthographic camera, and a tube skinned by a
four-bone chain (default and fixed-normal lighting), the sphere with two shape keys and the
skinned tube with one under its skin, and the sphere without a vertex colour channel (lit and
shadeless), and the per-vertex light volume whose cells light their vertices with other lights
first (LightVolumeCell.useLights): draw order and every emitted float, bit for bit."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_c1_whole_path as G  # noqa: E402

FIXTURE = os.path.join(HERE, "golden", "c1_whole_path.npz")
CASES = ["c1", "c1_scaled_5lights", "c1_volume_vertex", "c1_volume_normal", "c1_volume_object", "c1_fog_add",
         "c1_fog_sub", "c1_fixed_normals", "c1_double_sided_nocull", "c1_unsorted_group"]
CPU_CASES = ["c1_pcorrect", "c1_snap", "c1_unlit", "c1_ortho", "c1_ortho_pcorrect", "skinned_tube",
             "skinned_tube_fixed", "c1_shape_keys", "skinned_tube_keyed", "c1_no_colors", "c1_no_colors_shadeless",
             "c1_volume_nested"]  # the oracle only (the GPU's parity for these
# camera options is checked against the oracle by the feature-scene tests)
ALL = CASES + CPU_CASES


@pytest.fixture(scope="module")
def fixture():
    return np.load(FIXTURE)


@pytest.fixture(scope="module")
def scenes_():
    return {**G.cases(), **G.cpu_cases()}


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name", ALL)
def test_restatement_reproduces_fixture(fixture, scenes_, name):
    S = G.scene_inputs(scenes_[name])
    assert bytes(fixture[f"{name}_digest"]).hex() == G.input_digest(S), "scene inputs changed"
    order, xyuv, rgba, depth, custom0 = G.render(S, want_custom0=True)
    assert len(order) > 200
    assert np.array_equal(order, fixture[f"{name}_order"])
    for k, v in (("xyuv", xyuv), ("rgba", rgba), ("depth", depth), ("custom0", custom0)):
        if v is not None:
            assert np.array_equal(_bits(v), _bits(fixture[f"{name}_{k}"])), k


@pytest.mark.parametrize("name", ALL)
def test_cpp_oracle_matches_numpy_restatement(built, fixture, scenes_, name):
    from oracle import pyoracle
    sd = scenes_[name]
    ref = pyoracle.render(sd, sd.camera)
    assert ref.culled_models == 0
    assert np.array_equal(ref.tri_index.astype(np.uint32), fixture[f"{name}_order"]), "draw order"
    for k in ("xyuv", "rgba", "depth"):
        assert np.array_equal(_bits(getattr(ref, k)), _bits(fixture[f"{name}_{k}"])), k
    if f"{name}_custom0" in fixture:
        assert np.array_equal(_bits(ref.custom0), _bits(fixture[f"{name}_custom0"])), "custom0"


def test_scaled_case_exercises_the_added_lights(scenes_):
    """The two added point lights change colours of the scaled case (the near one lights part of
    the sphere; the far one is dropped by the model-level range skip), so the fixture covers a
    multi-light sum and the skip."""
    S = G.scene_inputs(scenes_["c1_scaled_5lights"])
    full = G.render(S)[2]
    three = G.render(dict(S, lights=S["lights"][:3]))[2]
    four = G.render(dict(S, lights=S["lights"][:4]))[2]
    assert (full != three).any(-1).sum() > 100
    assert np.array_equal(_bits(full), _bits(four))


@pytest.mark.parametrize("name", ["c1_volume_vertex", "c1_volume_normal", "c1_volume_object"])
def test_volume_cases_exercise_the_volume(scenes_, name):
    """The light volume changes the colours of most visible corners in each shading mode (per
    vertex, per vertex with the normal, per object), so the fixture covers the cell grid, the
    index rounding, the offset and bias and each mode's containment test."""
    S = G.scene_inputs(scenes_[name])
    with_volume = G.render(S)[2]
    without = G.render(dict(S, lights=S["lights"][:5]))[2]
    assert (with_volume != without).any(-1).sum() > 900


@pytest.mark.parametrize("name", ["c1_fog_add", "c1_fog_sub"])
def test_fog_cases_change_every_corner(scenes_, name):
    """Fog on without depth rendering changes the colour of every visible corner."""
    S = G.scene_inputs(scenes_[name])
    fogged = G.render(S)[2]
    plain = G.render(dict(S, fog_on=False, render_depth=True))[2]
    assert (fogged != plain).any(-1).all()


def test_material_and_group_cases_differ_from_the_base(scenes_):
    """Fixed normals change the lit colours; double-sided lighting without backface culling keeps
    all 960 triangles, front to back; the unsorted LightGroup case keeps triangle order and drops
    two lights."""
    base = G.render(G.scene_inputs(scenes_["c1_scaled_5lights"]))
    fixed = G.render(G.scene_inputs(scenes_["c1_fixed_normals"]))
    assert np.array_equal(fixed[0], base[0]) and (fixed[2] != base[2]).any(-1).sum() > 300
    both = G.render(G.scene_inputs(scenes_["c1_double_sided_nocull"]))
    assert len(both[0]) == 960
    grp = G.render(G.scene_inputs(scenes_["c1_unsorted_group"]))
    assert np.array_equal(grp[0], np.sort(grp[0])) and not np.array_equal(grp[0], base[0])
    assert len(G.scene_inputs(scenes_["c1_unsorted_group"])["lights"]) == 3


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_numpy_restatement(ctx, fixture, scenes_, name):
    from tetra3d_gb300 import abi
    sd = scenes_[name]
    sid = ctx.upload(sd)
    try:
        for mode in (abi.MODE_PLAIN, abi.MODE_BATCHED):
            ctx.render(sid, sd.camera, mode=mode)
            got = ctx.download()
            assert got.xyuv.shape[0] == len(fixture[f"{name}_order"])
            for k in ("xyuv", "rgba", "depth"):
                assert np.array_equal(_bits(getattr(got, k)), _bits(fixture[f"{name}_{k}"])), (mode, k)
    finally:
        ctx.release(sid)


def test_skinned_case_exercises_the_skin(scenes_):
    """The skinned tube differs from the same tube drawn unskinned, and its weights hold blends,
    exact 1.0 weights and 1.0 weights after a partial one (where Model.skinVertex stops)."""
    S = G.scene_inputs(scenes_["skinned_tube"])
    skinned = G.render(S)
    plain = G.render(dict(S, skinned=False))
    assert len(skinned[0]) == 1920 and not np.array_equal(_bits(skinned[1]), _bits(plain[1]))
    w = S["weights"]
    assert ((w > 0) & (w < 1)).any(1).sum() > 100 and (w == 1).any(1).sum() > 10
    late = [(0 < w[v, :k]).any() and w[v, k] == 1 for v in range(len(w)) for k in range(1, 4)]
    assert any(late)


@pytest.mark.parametrize("name", ["c1_shape_keys", "skinned_tube_keyed"])
def test_shape_key_cases_move_the_vertices(scenes_, name):
    """The keys change what the stage emits (the triangle centres and dimensions stay on the
    base mesh, the vertices move)."""
    S = G.scene_inputs(scenes_[name])
    keyed = G.render(S)
    base = G.render(dict(S, shape_weights=None))
    assert len(keyed[0]) != len(base[0]) or not np.array_equal(_bits(keyed[1]), _bits(base[1]))


def test_nested_case_uses_the_cell_lights(scenes_):
    """The cells' useLights change the colours of hundreds of corners."""
    S = G.scene_inputs(scenes_["c1_volume_nested"])
    nested = G.render(S)[2]
    plain = G.render(dict(S, cell_uses=None))[2]
    assert (nested != plain).any(-1).sum() > 300


FRAMES = ["six_spheres", "six_spheres_transparent", "batch6", "two_parts"]
CULLED = {"six_spheres": 2, "six_spheres_transparent": 2, "batch6": 1, "two_parts": 0}


@pytest.mark.parametrize("name", FRAMES)
def test_frame_restatement_reproduces_fixture(fixture, name):
    import hashlib
    sd = G.frame_cases()[name]
    digest = hashlib.sha256("".join(G.input_digest(G.scene_inputs(sd, m)) for m in range(sd.nmodels)).encode())
    assert bytes(fixture[f"{name}_digest"]).hex() == digest.hexdigest(), "scene inputs changed"
    parts = G.render_frame(sd)
    assert np.array_equal(np.array([p[0] for p in parts], np.uint32), fixture[f"{name}_models"])
    assert np.array_equal(np.array([p[5] for p in parts], np.uint32), fixture[f"{name}_parts"])
    assert np.array_equal(np.array([len(p[1]) for p in parts], np.uint32), fixture[f"{name}_counts"])
    assert np.array_equal(np.concatenate([p[1] for p in parts]).astype(np.uint32), fixture[f"{name}_order"])
    for k, i in (("xyuv", 2), ("rgba", 3), ("depth", 4)):
        assert np.array_equal(_bits(np.concatenate([p[i] for p in parts])), _bits(fixture[f"{name}_{k}"])), k


@pytest.mark.parametrize("name", FRAMES)
def test_cpp_oracle_matches_frame_restatement(built, fixture, name):
    """Six models of one scene (two of them transparent in the second frame; four members of a
    dynamic batch in the third; a mesh cut into an opaque and a transparent part in the fourth):
    the oracle's render pairs in draw order (solids in model and part order,
    a batch's members far to near in its owner's place, then transparents far to near), the
    models the frustum test drops empty, and every other pair's triangles and floats equal to the
    restatement's."""
    from oracle import pyoracle
    sd = G.frame_cases()[name]
    ref = pyoracle.render(sd, sd.camera)
    assert ref.culled_models == CULLED[name]
    assert np.array_equal(np.array([s["model"] for s in ref.segments], np.uint32), fixture[f"{name}_models"])
    assert np.array_equal(np.array([s["part"] for s in ref.segments], np.uint32), fixture[f"{name}_parts"])
    assert np.array_equal(np.array([s["count"] for s in ref.segments], np.uint32), fixture[f"{name}_counts"])
    assert np.array_equal(ref.tri_index.astype(np.uint32), fixture[f"{name}_order"]), "draw order"
    for k in ("xyuv", "rgba", "depth"):
        assert np.array_equal(_bits(getattr(ref, k)), _bits(fixture[f"{name}_{k}"])), k
