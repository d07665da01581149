"""TEST INFRASTRUCTURE ONLY: ctypes front end of the oracle (oracle/t3d_oracle.cpp).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; never by the product path. PARITY UNPINNED by reference tests (see
t3d_oracle.h).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from tetra3d_gb300 import abi  # noqa: E402  (struct layouts shared with include/t3d.h)

LIB_PATH = os.path.join(HERE, "_build", "libt3d_oracle.so")


class OracleOut(C.Structure):
    _fields_ = [("max_segments", C.c_uint32), ("num_segments", C.c_uint32),
                ("seg_model", C.POINTER(C.c_uint32)), ("seg_part", C.POINTER(C.c_uint32)),
                ("seg_base", C.POINTER(C.c_uint32)), ("seg_capacity", C.POINTER(C.c_uint32)),
                ("seg_count", C.POINTER(C.c_uint32)), ("max_tris", C.c_uint64), ("total_slots", C.c_uint64),
                ("visible_tris", C.c_uint64), ("tri_index", C.POINTER(C.c_uint32)), ("xyuv", C.c_void_p),
                ("rgba", C.c_void_p), ("depth", C.c_void_p), ("culled_models", C.c_uint32), ("reserved", C.c_uint32),
                ("seg_draw", C.POINTER(C.c_uint32)), ("seg_draw_transparent", C.POINTER(C.c_uint32)),
                ("custom0", C.c_void_p)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from oracle import build_oracle
            build_oracle.build()
        lib = C.CDLL(LIB_PATH)
        for name in ("t3d_oracle_render_f32", "t3d_oracle_render_f64"):
            fn = getattr(lib, name)
            fn.restype = C.c_int
            fn.argtypes = [C.POINTER(abi.SceneDesc), C.POINTER(abi.CameraDesc), C.POINTER(C.c_uint64), C.c_uint32,
                           C.c_uint32, C.POINTER(OracleOut)]
        f = C.POINTER(C.c_float)
        lib.t3d_oracle_mat_mult.argtypes = [f, f, f]
        lib.t3d_oracle_mat_inverted.argtypes = [f, f]
        lib.t3d_oracle_mat_rotate.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, f]
        lib.t3d_oracle_mat_decompose.argtypes = [f, f, f, f]
        lib.t3d_oracle_quat_to_mat.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, f]
        lib.t3d_oracle_vec_unit.argtypes = [f, f]
        for n in ("t3d_oracle_mat_mult", "t3d_oracle_mat_inverted", "t3d_oracle_mat_rotate",
                  "t3d_oracle_mat_decompose", "t3d_oracle_quat_to_mat", "t3d_oracle_vec_unit"):
            getattr(lib, n).restype = None
        _lib = lib
    return _lib


class OracleFrame:
    def __init__(self, segs, tri_index, xyuv, rgba, depth, culled, custom0=None):
        self.segments = segs      # list of dicts model, part, base, capacity, count (draw order)
        self.tri_index = tri_index  # (n,) mesh-absolute triangle per visible triangle, in emit order
        self.xyuv, self.rgba, self.depth = xyuv, rgba, depth
        self.culled_models = culled
        self.custom0 = custom0    # (n, 3) 1 / w per corner under perspective-corrected mapping, else None

    @property
    def visible_tris(self):
        return int(self.tri_index.shape[0])


def render(scene_data, cam, light_mask=None, animate_frames=0, threads=1, f64=False):
    """Runs the CPU restatement of Camera.Render on a SceneData and returns an OracleFrame
    with the visible triangles compacted in draw order (same layout as the GPU download)."""
    lib = load()
    sd = scene_data.desc()
    nseg_max = sum(len(scene_data.meshes[int(m)].parts) for m in scene_data.mv["mesh"]) + 1
    slots = max(1, scene_data.total_tris())
    while True:
        frame, rc, need = _render_into(lib, sd, cam, light_mask, animate_frames, threads, f64, nseg_max, slots)
        if rc == 0:
            return frame
        if need <= slots:  # not a capacity problem
            raise RuntimeError(f"oracle render failed: {rc}")
        slots = need  # auto-subdivided meshes list more triangles than the scene holds


def _render_into(lib, sd, cam, light_mask, animate_frames, threads, f64, nseg_max, slots):
    dt = np.float64 if f64 else np.float32
    seg = {k: np.zeros(nseg_max, np.uint32) for k in ("model", "part", "base", "capacity", "count", "draw",
                                                       "draw_transparent")}
    tri = np.zeros(slots, np.uint32)
    xyuv = np.zeros((slots, 3, 4), dt)
    rgba = np.zeros((slots, 3, 4), dt)
    depth = np.zeros((slots, 3), dt)
    custom0 = np.zeros((slots, 3), dt) if cam.perspective_corrected else None
    o = OracleOut()
    o.max_segments = nseg_max
    u = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint32))
    o.seg_model, o.seg_part, o.seg_base = u(seg["model"]), u(seg["part"]), u(seg["base"])
    o.seg_capacity, o.seg_count = u(seg["capacity"]), u(seg["count"])
    o.seg_draw, o.seg_draw_transparent = u(seg["draw"]), u(seg["draw_transparent"])
    o.max_tris = slots
    o.tri_index = u(tri)
    o.xyuv, o.rgba, o.depth = xyuv.ctypes.data, rgba.ctypes.data, depth.ctypes.data
    o.custom0 = custom0.ctypes.data if custom0 is not None else None
    mask = None
    if light_mask is not None:
        m = (C.c_uint64 * 2)(light_mask & ((1 << 64) - 1), (light_mask >> 64) & ((1 << 64) - 1))
        mask = C.cast(m, C.POINTER(C.c_uint64))
    fn = lib.t3d_oracle_render_f64 if f64 else lib.t3d_oracle_render_f32
    rc = fn(C.byref(sd), C.byref(cam), mask, animate_frames, threads, C.byref(o))
    if rc != 0:
        return None, rc, int(o.total_slots)
    n = o.num_segments
    segs = [dict(model=int(seg["model"][i]), part=int(seg["part"][i]), base=int(seg["base"][i]),
                 capacity=int(seg["capacity"][i]), count=int(seg["count"][i]), draw=int(seg["draw"][i]),
                 draw_transparent=int(seg["draw_transparent"][i])) for i in range(n)]
    sel = np.concatenate([np.arange(s["base"], s["base"] + s["count"]) for s in segs] or [np.zeros(0, np.int64)])
    sel = sel.astype(np.int64)
    return OracleFrame(segs, tri[sel], xyuv[sel], rgba[sel], depth[sel], o.culled_models,
                       custom0[sel] if custom0 is not None else None), 0, slots


class Renderer:
    """The oracle's Camera.Render of one scene and camera with its output arrays allocated once,
    for timing: like the reference's render loop, which reuses its scratch and vertex lists frame
    after frame, a call does the render alone (no allocation, no compaction of the output)."""

    def __init__(self, scene_data, cam, light_mask=None, f64=False):
        self.lib = load()
        self.scene_data = scene_data  # the descriptor points into its arrays
        self.sd = scene_data.desc()
        self.cam = cam
        self.dt = np.float64 if f64 else np.float32
        self.nseg_max = sum(len(scene_data.meshes[int(m)].parts) for m in scene_data.mv["mesh"]) + 1
        self.mask = None
        if light_mask is not None:
            self._m = (C.c_uint64 * 2)(light_mask & ((1 << 64) - 1), (light_mask >> 64) & ((1 << 64) - 1))
            self.mask = C.cast(self._m, C.POINTER(C.c_uint64))
        self.fn = self.lib.t3d_oracle_render_f64 if f64 else self.lib.t3d_oracle_render_f32
        self._alloc(max(1, scene_data.total_tris()))

    def _alloc(self, slots):
        dt, nseg_max = self.dt, self.nseg_max
        self.slots = slots
        self.count = np.zeros(nseg_max, np.uint32)
        self.arrays = [np.zeros(nseg_max, np.uint32) for _ in range(6)] + [np.zeros(slots, np.uint32)]
        self.out = [np.zeros((slots, 3, 4), dt), np.zeros((slots, 3, 4), dt), np.zeros((slots, 3), dt)]
        self.custom0 = np.zeros((slots, 3), dt) if self.cam.perspective_corrected else None
        o = OracleOut()
        o.max_segments = nseg_max
        u = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint32))
        a = self.arrays
        o.seg_model, o.seg_part, o.seg_base, o.seg_capacity = u(a[0]), u(a[1]), u(a[2]), u(a[3])
        o.seg_count = u(self.count)
        o.seg_draw, o.seg_draw_transparent = u(a[4]), u(a[5])
        o.max_tris = slots
        o.tri_index = u(a[6])
        o.xyuv, o.rgba, o.depth = self.out[0].ctypes.data, self.out[1].ctypes.data, self.out[2].ctypes.data
        o.custom0 = self.custom0.ctypes.data if self.custom0 is not None else None
        self.o = o

    def render(self, animate_frames=0, threads=1):
        """Renders into the arrays; returns the visible triangles."""
        rc = self.fn(C.byref(self.sd), C.byref(self.cam), self.mask, animate_frames, threads, C.byref(self.o))
        if rc != 0 and int(self.o.total_slots) > self.slots:
            # auto-subdivided meshes list more triangles than the scene holds: grow once, render again
            self._alloc(int(self.o.total_slots))
            rc = self.fn(C.byref(self.sd), C.byref(self.cam), self.mask, animate_frames, threads, C.byref(self.o))
        if rc != 0:
            raise RuntimeError(f"oracle render failed: {rc}")
        return int(self.count[:self.o.num_segments].sum())


def mat_inverted(m):
    lib = load()
    a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
    out = np.zeros(16, np.float32)
    lib.t3d_oracle_mat_inverted(a.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)))
    return out.reshape(4, 4)


def mat_mult(a, b):
    lib = load()
    a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(16))
    b = np.ascontiguousarray(np.asarray(b, np.float32).reshape(16))
    out = np.zeros(16, np.float32)
    p = lambda x: x.ctypes.data_as(C.POINTER(C.c_float))
    lib.t3d_oracle_mat_mult(p(a), p(b), p(out))
    return out.reshape(4, 4)


def mat_rotate(x, y, z, angle):
    lib = load()
    out = np.zeros(16, np.float32)
    lib.t3d_oracle_mat_rotate(x, y, z, angle, out.ctypes.data_as(C.POINTER(C.c_float)))
    return out.reshape(4, 4)


def quat_to_mat(x, y, z, w):
    lib = load()
    out = np.zeros(16, np.float32)
    lib.t3d_oracle_quat_to_mat(x, y, z, w, out.ctypes.data_as(C.POINTER(C.c_float)))
    return out.reshape(4, 4)


def vec_unit(v):
    lib = load()
    a = np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))
    out = np.zeros(3, np.float32)
    lib.t3d_oracle_vec_unit(a.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def is_transparent(model_row, mat):
    """Model.isTransparent for one mesh part (model.go:1086-1107, material.go:192-207)."""
    F = np.float32
    if mat["present"]:
        mat_t = (mat["transparency_mode"] == abi.TRANSPARENCY_TRANSPARENT or not mat["blend_source_over"]
                 or (mat["transparency_mode"] == abi.TRANSPARENCY_AUTO and F(mat["color"][3]) < F(0.999)))
        model_t = mat["transparency_mode"] != abi.TRANSPARENCY_OPAQUE and F(model_row["color"][3]) < F(0.999)
        return bool(mat_t or model_t)
    return bool(F(model_row["color"][3]) < F(0.999))


class OracleTextures(C.Structure):
    _fields_ = [("flush_texture", C.POINTER(C.c_uint32)), ("flush_flags", C.POINTER(C.c_uint32)),
                ("flush_scale", C.POINTER(C.c_float)), ("ntex", C.c_uint32), ("tex_offset", C.POINTER(C.c_uint32)),
                ("tex_w", C.POINTER(C.c_int32)), ("tex_h", C.POINTER(C.c_int32)), ("texels", C.POINTER(C.c_uint32))]


def flush_material(scene_data, seg):
    """The material a flush draws with: a dynamic batch's members flush with the batch pair's
    part (camera.go:2075-2100, flush at :1829-1845), anything else with its own."""
    md = scene_data.mv[seg["model"]]
    if int(md["batched"]):
        owner = scene_data.mv[int(md["batch_owner"])]
        return scene_data.meshes[int(owner["mesh"])].parts[int(md["batch_part"])]["mat"]
    return scene_data.meshes[int(md["mesh"])].parts[seg["part"]]["mat"]


def texture_state(mat):
    """(texture, flags, (scale_w, scale_h)) of a flush material, as the device reads them."""
    if not mat.get("present", 1):
        return 0, 0, (0.0, 0.0)
    flags = (1 if mat.get("texture_filter", 0) else 0) | (2 if mat.get("texture_map_mode", 0) == 1 else 0) | \
        (4 if mat["transparency_mode"] == abi.TRANSPARENCY_ALPHA_CLIP else 0)
    return int(mat.get("texture", 0)), flags, tuple(mat.get("texture_map_scale", (1.0, 1.0)))


def raster(frame, scene_data, cam, fog_curve=0, dither_size=0.0, fogless=0, transparent=None, textures=None,
           flush_tex=None):
    """Oracle of t3d_frame_raster for a one-job frame (an OracleFrame or a downloaded frame, both
    compacted in draw order with .segments). Returns (colour, depth) RGBA8 (height, width, 4).
    `transparent` (one flag per segment) replaces the flags derived from scene_data; `textures`
    is the texture table (premultiplied RGBA8 (height, width, 4) arrays, as given to
    t3d_raster_set_textures); `flush_tex` (one (texture, flags, (scale_w, scale_h)) per segment)
    replaces the texture state derived from the flush materials."""
    lib = load()
    fn = lib.t3d_oracle_raster
    u32p, f32p = C.POINTER(C.c_uint32), C.POINTER(C.c_float)
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(abi.CameraDesc), C.c_int32, C.c_float, C.c_int32, C.c_uint32, f32p, f32p, f32p, u32p,
                   C.POINTER(C.c_uint8), C.POINTER(OracleTextures), u32p, u32p, f32p]
    n = int(frame.xyuv.shape[0])
    pair = np.zeros(max(1, n), np.uint32)
    given = transparent
    nseg = max(1, len(frame.segments))
    transparent = np.zeros(nseg, np.uint8)
    ftex, fflags, fscale = np.zeros(nseg, np.uint32), np.zeros(nseg, np.uint32), np.zeros((nseg, 2), np.float32)
    b = 0
    flush = -1
    for k, s in enumerate(frame.segments):
        # the pairs of one dynamic batch are one flush (one depth composite)
        if k == 0 or "draw" not in s or s["draw"] != frame.segments[k - 1]["draw"]:
            flush += 1
            if flush_tex is not None:
                st = flush_tex[k]
            elif textures is not None and scene_data is not None:
                st = texture_state(flush_material(scene_data, s))
            else:
                st = (0, 0, (0.0, 0.0))
            ftex[flush], fflags[flush], fscale[flush] = st[0], st[1], st[2]
        pair[b:b + s["count"]] = flush
        b += s["count"]
        if given is not None:
            transparent[flush] = bool(given[k])
        elif "draw_transparent" in s:
            transparent[flush] = bool(s["draw_transparent"])
        else:
            md = scene_data.mv[s["model"]]
            mat = scene_data.meshes[int(md["mesh"])].parts[s["part"]]["mat"]
            transparent[flush] = is_transparent(md, mat)
    xyuv = np.ascontiguousarray(frame.xyuv, np.float32).reshape(-1)
    rgba = np.ascontiguousarray(frame.rgba, np.float32).reshape(-1)
    depth = np.ascontiguousarray(frame.depth, np.float32).reshape(-1)
    custom0 = None
    if cam.perspective_corrected:
        assert getattr(frame, "custom0", None) is not None, "perspective-corrected frame without Custom0"
        custom0 = np.ascontiguousarray(frame.custom0, np.float32).reshape(-1)
    W, H = cam.width, cam.height
    col = np.zeros(W * H, np.uint32)
    dep = np.zeros(W * H, np.uint32)
    texs = list(textures or [])
    sizes = [(int(t.shape[1]), int(t.shape[0])) for t in texs]
    offs = np.zeros(max(1, len(texs)), np.uint32)
    offs[1:len(texs)] = np.cumsum([w * h for w, h in sizes])[:-1] if len(texs) > 1 else []
    tw = np.array([w for w, _ in sizes] or [0], np.int32)
    th = np.array([h for _, h in sizes] or [0], np.int32)
    texels = np.concatenate([np.ascontiguousarray(t, np.uint8).reshape(-1, 4).view(np.uint32).reshape(-1)
                             for t in texs]) if texs else np.zeros(1, np.uint32)
    assert np.all(ftex[:flush + 1] <= len(texs)), "a flush names a texture beyond the table"
    ts = OracleTextures(ftex.ctypes.data_as(u32p), fflags.ctypes.data_as(u32p), fscale.ctypes.data_as(f32p), len(texs),
                        offs.ctypes.data_as(u32p), tw.ctypes.data_as(C.POINTER(C.c_int32)),
                        th.ctypes.data_as(C.POINTER(C.c_int32)), texels.ctypes.data_as(u32p))
    rc = fn(C.byref(cam), fog_curve, dither_size, fogless, n, xyuv.ctypes.data_as(f32p), rgba.ctypes.data_as(f32p),
            depth.ctypes.data_as(f32p), pair.ctypes.data_as(u32p), transparent.ctypes.data_as(C.POINTER(C.c_uint8)),
            C.byref(ts), col.ctypes.data_as(u32p), dep.ctypes.data_as(u32p),
            custom0.ctypes.data_as(f32p) if custom0 is not None else None)
    if rc != 0:
        raise RuntimeError(f"oracle raster failed: {rc}")
    return col.view(np.uint8).reshape(H, W, 4), dep.view(np.uint8).reshape(H, W, 4)
