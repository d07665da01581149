"""t3d_render_part_noalloc: the render entry point for callers that cannot allocate.

Engines that own the device memory budget, or real-time render threads where a
cudaMalloc would stall the frame, render one model part through this call with
their own input and output buffers; every intermediate lives in a fixed array
inside the library. This test renders the same parts through that call and
through the regular context API (t3d_scene_upload + t3d_render) and requires
identical output bits, twice in a row (the shared array keeps the previous
call's contents, so the second call checks that nothing leaks between calls).
It runs last so that a failure here leaves every other test already run; it
also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from tetra3d_gb300 import abi, scenes
from tests.parity import bits

pytestmark = pytest.mark.gpu


def _reference(ctx, sd, mesh):
    """One-model scene through the regular API; returns (xyuv, rgba, depth) of model 0."""
    sid = ctx.upload(sd)
    try:
        ctx.render(sid, sd.camera)
        f = ctx.download()
    finally:
        ctx.release(sid)
    return f.xyuv, f.rgba, f.depth


def _noalloc(lib, sd, torch):
    me = sd.meshes[0]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pos, nrm, uv = dev(me.positions), dev(me.normals), dev(me.uvs)
    col = dev(me.colors) if me.colors is not None else None
    idx = dev(me.indices.astype(np.int32))
    part = me.parts[0]
    n = part["tri_count"]
    out_xyuv = torch.full((n, 3, 4), float("nan"), device="cuda")
    out_rgba = torch.full((n, 3, 4), float("nan"), device="cuda")
    out_depth = torch.full((n, 3), float("nan"), device="cuda")
    out_count = torch.zeros(1, dtype=torch.int32, device="cuda")
    lst = sd.lists[0] if sd.mv["light_list"][0] < 0 else sd.lists[int(sd.mv["light_list"][0])]
    lights = (abi.LightDesc * max(1, len(lst)))(*[sd.lights[i] for i in lst])
    a = abi.NoallocArgs()
    a.positions, a.normals, a.uvs = pos.data_ptr(), nrm.data_ptr(), uv.data_ptr()
    a.colors = col.data_ptr() if col is not None else None
    a.indices = idx.data_ptr()
    a.volume_cells = None
    a.out_xyuv, a.out_rgba, a.out_depth = out_xyuv.data_ptr(), out_rgba.data_ptr(), out_depth.data_ptr()
    a.out_count = out_count.data_ptr()
    a.model = C.pointer(sd.models[0])
    a.lights = C.cast(lights, C.POINTER(abi.LightDesc))
    a.camera = C.pointer(sd.camera)
    a.num_vertices, a.num_triangles = me.nverts, me.ntris
    a.tri_start, a.tri_count = part["tri_start"], n
    a.num_lights = len(lst)
    a.dim_min[:] = [float(x) for x in me.positions.min(0)]
    a.dim_max[:] = [float(x) for x in me.positions.max(0)]
    for k, v in part["mat"].items():
        if k == "color":
            a.mat.color[:] = [float(c) for c in v]
        elif k == "billboard_lock":
            a.mat.billboard_lock[:] = [int(c) for c in v]
        else:
            setattr(a.mat, k, v)
    torch.cuda.synchronize()
    rc = lib.t3d_render_part_noalloc(0, C.byref(a), None)
    assert rc == abi.T3D_OK, a.error.decode()
    k = int(out_count.item())
    return out_xyuv[:k].cpu().numpy(), out_rgba[:k].cpu().numpy(), out_depth[:k].cpu().numpy()


def _grid_scene(seed):
    """A single lit grid model with enough triangles for several tiles (the multi-tile path)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    me = scenes.grid_mesh(64, 64, 8.0, 8.0, lambda X, Z: 0.3 * np.sin(X) * np.cos(Z), x0=-4.0, z0=-4.0)
    me.colors = rng.uniform(0.5, 1.0, (me.nverts, 4)).astype(np.float32)
    lights = [scenes.light(abi.LIGHT_AMBIENT, energy=0.2),
              scenes.light(abi.LIGHT_POINT, color=(1.0, 0.8, 0.6), energy=3.0, rng_=12.0, pos=(1, 3, -2)),
              scenes.light(abi.LIGHT_DIRECTIONAL, energy=0.7,
                           rot=scenes.look_rotation(scenes.unit3(np.array([0.2, 1.0, 0.4], np.float32))))]
    sd = scenes.SceneData([me], 1, lights, [[0, 1, 2]], name="grid64")
    rot = scenes.rotate(1, 0, 0, scenes.deg2rad(30.0))  # tilted towards the camera
    scenes.set_models_trs(sd, 0, [(0, -1, -9)], [(1, 1, 1)], rot[None])
    sd.camera = scenes.camera(w=1280, h=720, fov=70.0)
    return sd


@pytest.mark.parametrize("which", ["uv_sphere", "grid", "billboard"])
def test_noalloc_matches_context_api_twice(ctx, which):
    torch = pytest.importorskip("torch")
    sd = scenes.uv_sphere_scene(5) if which != "grid" else _grid_scene(6)
    if which == "billboard":  # the turned part runs the kernel's altered-vertex loop
        sd.meshes[0].parts[0]["mat"].update(billboard=1, billboard_lock=(0, 1, 0),
                                             billboard_depth=abi.DEPTH_UNBILLBOARDED)
    ref = _reference(ctx, sd, sd.meshes[0])
    assert ref[0].shape[0] > 0
    for call in range(2):
        got = _noalloc(ctx.lib, sd, torch)
        for name, g, r in zip(("xyuv", "rgba", "depth"), got, ref):
            assert g.shape == r.shape, f"call {call}: {name} {g.shape} vs {r.shape}"
            assert np.array_equal(bits(g), bits(r)), f"call {call}: {name} differs from the context API"


def test_noalloc_rejects_oversize(ctx):
    a = abi.NoallocArgs()
    sd = scenes.uv_sphere_scene(5)
    a.model = C.pointer(sd.models[0])
    a.camera = C.pointer(sd.camera)
    a.positions = a.normals = a.uvs = a.indices = 1  # never dereferenced: rejected before any device work
    a.out_xyuv = a.out_rgba = a.out_depth = a.out_count = 1
    a.num_vertices, a.num_triangles, a.tri_count = 1 << 20, 10, 10
    rc = ctx.lib.t3d_render_part_noalloc(0, C.byref(a), None)
    assert rc == abi.T3D_E_INVAL
    assert b"no-alloc limits" in a.error


def test_noalloc_reports_empty_mesh_and_part_outside(ctx):
    sd = scenes.uv_sphere_scene(5)
    for nv, nt, start, cnt, want in ((0, 10, 0, 10, b"empty mesh"), (100, 10, 8, 5, b"outside")):
        a = abi.NoallocArgs()
        a.model = C.pointer(sd.models[0])
        a.camera = C.pointer(sd.camera)
        a.positions = a.normals = a.uvs = a.indices = 1  # rejected before any device work
        a.out_xyuv = a.out_rgba = a.out_depth = a.out_count = 1
        a.num_vertices, a.num_triangles, a.tri_start, a.tri_count = nv, nt, start, cnt
        assert ctx.lib.t3d_render_part_noalloc(0, C.byref(a), None) == abi.T3D_E_INVAL
        assert want in a.error, a.error


def test_context_with_larger_tiles_renders_after_noalloc_calls(ctx):
    """The frame kernel's shared-memory limit is one attribute for the whole process: a
    context tuned for 4096-triangle tiles (more shared memory than the allocation-free
    entry uses) still launches after allocation-free calls."""
    torch = pytest.importorskip("torch")
    sd = _grid_scene(8)
    _noalloc(ctx.lib, sd, torch)
    ctx.set_tuning(tile_tris=4096)
    try:
        sid = ctx.upload(sd)
        try:
            ctx.render(sid, sd.camera)
            ref = ctx.download()
            _noalloc(ctx.lib, sd, torch)
            ctx.render(sid, sd.camera)
            got = ctx.download()
        finally:
            ctx.release(sid)
        assert got.visible_tris == ref.visible_tris > 0
        assert np.array_equal(bits(got.xyuv), bits(ref.xyuv))
    finally:
        ctx.set_tuning(tile_tris=2048)
