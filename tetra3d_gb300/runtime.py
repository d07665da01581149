"""Python host wrapper over libt3d.so (the GB300 vertex stage).

Context mirrors the reference's per-frame flow: upload a Scene once, then call
render(camera) per frame (Camera.Render, camera.go:1269), sync, and read the
emitted triangle stream. All compute runs in the CUDA library; this module only
marshals arguments.
"""
import ctypes as C

import numpy as np

from . import abi


class Frame:
    """Host copy of one rendered frame: visible triangles in draw order."""

    def __init__(self, xyuv, rgba, depth, segments, stats):
        self.xyuv = xyuv          # (n, 3, 4) float32 per corner DstX, DstY, SrcX, SrcY
        self.rgba = rgba          # (n, 3, 4) float32 colour vertex colour
        self.depth = depth        # (n, 3) float32 depth vertex colour
        self.segments = segments  # list of dicts: job, model, part, base, capacity, count
        self.stats = stats

    @property
    def visible_tris(self):
        return int(self.stats.visible_tris)


class Context:
    def __init__(self, device=0, lib=None):
        self.lib = lib or abi.load()
        h = C.c_void_p()
        rc = self.lib.t3d_create(device, C.byref(h))
        if rc != abi.T3D_OK:
            raise abi.T3DError(rc, f"t3d_create(device={device}) failed")
        self.h = h
        self.scenes = {}

    def _check(self, rc, what):
        if rc != abi.T3D_OK:
            raise abi.T3DError(rc, f"{what}: {self.lib.t3d_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            self.lib.t3d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning(self, tile_tris=0, vertex_chunk=0, block_threads=0):
        self._check(self.lib.t3d_set_tuning(self.h, tile_tris, vertex_chunk, block_threads), "set_tuning")

    def set_meshlets(self, enable):
        """Meshlet route for plain render pairs (default on); off sends every pair through the
        per-vertex record path. The emitted stream is the same either way."""
        self._check(self.lib.t3d_set_meshlets(self.h, int(bool(enable))), "set_meshlets")

    def set_split_phases(self, mode):
        """Launch shape: 1 (default) one persistent launch per phase, 0 a batched frame as one
        cooperative launch with grid barriers between the phases. The stream is the same."""
        self._check(self.lib.t3d_set_split_phases(self.h, int(mode)), "set_split_phases")

    def set_wait_limit(self, polls):
        """Polls a bounded device wait makes before the frame gives up (0: the default)."""
        self._check(self.lib.t3d_set_wait_limit(self.h, int(polls)), "set_wait_limit")

    def upload(self, scene_data):
        sd = scene_data.desc()
        sid = C.c_uint32()
        self._check(self.lib.t3d_scene_upload(self.h, C.byref(sd), C.byref(sid)), "scene_upload")
        self.scenes[sid.value] = scene_data
        return sid.value

    def release(self, sid):
        self._check(self.lib.t3d_scene_release(self.h, sid), "scene_release")
        self.scenes.pop(sid, None)

    def set_models(self, sid, scene_data, first=0, n=None):
        n = scene_data.nmodels - first if n is None else n
        ptr = C.cast(C.byref(scene_data.models, first * C.sizeof(abi.ModelDesc)), C.POINTER(abi.ModelDesc))
        self._check(self.lib.t3d_scene_set_models(self.h, sid, first, ptr, n), "scene_set_models")

    def set_bones(self, sid, bones, first=0):
        """Bone influence matrices (n, 4, 4) of the scene's bones first..first+n."""
        b = np.ascontiguousarray(bones, np.float32).reshape(-1, 16)
        self._check(self.lib.t3d_scene_set_bones(self.h, sid, first, abi.fptr(b), b.shape[0]), "scene_set_bones")

    def set_lights(self, sid, scene_data, first=0, n=None):
        """Lights [first, first + n) of the scene from scene_data.lights."""
        n = scene_data.nlights - first if n is None else n
        ptr = C.cast(C.byref(scene_data.lights, first * C.sizeof(abi.LightDesc)), C.POINTER(abi.LightDesc))
        self._check(self.lib.t3d_scene_set_lights(self.h, sid, first, ptr, n), "scene_set_lights")

    def set_shape_weights(self, sid, mesh, weights):
        w = np.ascontiguousarray(weights, np.float32).reshape(-1)
        self._check(self.lib.t3d_scene_set_shape_weights(self.h, sid, mesh, abi.fptr(w), w.shape[0]),
                    "scene_set_shape_weights")

    def transforms(self, sid, n):
        out = np.zeros((n, 16), np.float32)
        self._check(self.lib.t3d_scene_get_transforms(self.h, sid, abi.fptr(out), n), "scene_get_transforms")
        return out.reshape(n, 4, 4)

    def render(self, sid, cam, mode=abi.MODE_BATCHED, animate=False, stream=None):
        self._check(self.lib.t3d_render(self.h, sid, C.byref(cam), mode, int(animate), stream), "render")

    def render_jobs(self, jobs, mode=abi.MODE_BATCHED, animate=False, stream=None):
        arr = (abi.JobDesc * len(jobs))(*jobs)
        self._check(self.lib.t3d_render_jobs(self.h, arr, len(jobs), mode, int(animate), stream), "render_jobs")

    def sync(self):
        st = abi.Stats()
        self._check(self.lib.t3d_frame_sync(self.h, C.byref(st)), "frame_sync")
        return st

    def readback(self):
        """Enqueues the read-back of the last frame's counts (collect() returns them)."""
        self._check(self.lib.t3d_frame_readback(self.h), "frame_readback")

    def collect(self):
        """Waits for the read-back started by readback() and returns that frame's stats."""
        st = abi.Stats()
        self._check(self.lib.t3d_frame_collect(self.h, C.byref(st)), "frame_collect")
        return st

    def segments(self):
        n = C.c_uint32()
        self._check(self.lib.t3d_frame_segments(self.h, None, 0, C.byref(n)), "frame_segments")
        arr = (abi.SegmentInfo * max(1, n.value))()
        self._check(self.lib.t3d_frame_segments(self.h, arr, n.value, C.byref(n)), "frame_segments")
        return [dict(job=s.job, model=s.model, part=s.part, base=s.base, capacity=s.capacity, count=s.count,
                     draw=s.draw, draw_transparent=s.draw_transparent) for s in arr[:n.value]]

    def download(self, stats=None):
        st = stats or self.sync()
        n = int(st.visible_tris)
        xyuv = np.zeros((max(1, n), 3, 4), np.float32)
        rgba = np.zeros((max(1, n), 3, 4), np.float32)
        depth = np.zeros((max(1, n), 3), np.float32)
        got = C.c_uint64()
        self._check(self.lib.t3d_frame_download(self.h, abi.fptr(xyuv), abi.fptr(rgba), abi.fptr(depth), n,
                                                C.byref(got)), "frame_download")
        return Frame(xyuv[:n], rgba[:n], depth[:n], self.segments(), st)

    def download_custom0(self, stats=None):
        """Custom0 (1 / w) of the last frame's visible corners, (n, 3) float32, same order as
        download(); the frame must use perspective-corrected texture mapping."""
        st = stats or self.sync()
        n = int(st.visible_tris)
        out = np.zeros((max(1, n), 3), np.float32)
        got = C.c_uint64()
        self._check(self.lib.t3d_frame_download_custom0(self.h, abi.fptr(out), n, C.byref(got)),
                    "frame_download_custom0")
        return out[:n]

    def counters(self):
        v, b = C.c_uint64(), C.c_uint64()
        self._check(self.lib.t3d_frame_counters(self.h, C.byref(v), C.byref(b)), "frame_counters")
        return v.value, b.value

    def view(self):
        v = abi.FrameView()
        self._check(self.lib.t3d_frame_view_get(self.h, C.byref(v)), "frame_view_get")
        return v

    def raster(self, job=0, fog_curve=0, dither_size=0.0, fogless=0, stream=None, download=True, shared_large_tris=0):
        """Rasterises one job of the last frame (the colour and depth passes of flush) and returns
        (colour, depth) RGBA8 images of shape (height, width, 4), premultiplied (None, None without
        download: the images stay on the device). `shared_large_tris` is the tuning knob of
        t3d_raster_opts (0 default, negative none)."""
        o = abi.RasterOpts(fog_curve, float(dither_size), fogless, int(shared_large_tris))
        self._check(self.lib.t3d_frame_raster(self.h, job, C.byref(o), stream), "frame_raster")
        if not download:
            return None, None
        w, h = C.c_int32(), C.c_int32()
        self._check(self.lib.t3d_frame_images(self.h, None, None, C.byref(w), C.byref(h)), "frame_images")
        col = np.zeros((h.value, w.value, 4), np.uint8)
        dep = np.zeros((h.value, w.value, 4), np.uint8)
        u8 = C.POINTER(C.c_uint8)
        self._check(self.lib.t3d_frame_images(self.h, col.ctypes.data_as(u8), dep.ctypes.data_as(u8), C.byref(w),
                                              C.byref(h)), "frame_images")
        return col, dep

    def set_textures(self, textures):
        """Replaces the raster texture table: premultiplied RGBA8 arrays of shape (height, width, 4);
        a material's `texture` k names entry k - 1."""
        keep = [np.ascontiguousarray(t, np.uint8) for t in textures]
        arr = (abi.TextureDesc * max(1, len(keep)))()
        for k, t in enumerate(keep):
            assert t.ndim == 3 and t.shape[2] == 4, "textures are (height, width, 4) RGBA8"
            arr[k] = abi.TextureDesc(t.ctypes.data_as(C.POINTER(C.c_uint8)), t.shape[1], t.shape[0])
        self._check(self.lib.t3d_raster_set_textures(self.h, arr, len(keep)), "raster_set_textures")

    def graph_capture(self, sid, cam, animate=True):
        self._check(self.lib.t3d_graph_capture(self.h, sid, C.byref(cam), int(animate)), "graph_capture")

    def graph_replay(self, frames=1, stream=None):
        self._check(self.lib.t3d_graph_replay(self.h, frames, stream), "graph_replay")


def job(sid, cam, light_mask=None):
    j = abi.JobDesc()
    j.scene = sid
    if light_mask is None:
        j.light_mask[0] = j.light_mask[1] = (1 << 64) - 1
    else:
        j.light_mask[0] = light_mask & ((1 << 64) - 1)
        j.light_mask[1] = (light_mask >> 64) & ((1 << 64) - 1)
    j.camera = cam
    return j


class Server:
    """Continuous-batching render server over a Context's resident scenes."""

    def __init__(self, ctx, hbm_budget_bytes=150 << 30, max_batch=64, streams=4, verify=True, max_pairs=None):
        self.ctx = ctx
        h = C.c_void_p()
        ctx._check(ctx.lib.t3d_server_create(ctx.h, hbm_budget_bytes, max_batch, streams, C.byref(h)), "server_create")
        self.h = h
        ctx.lib.t3d_server_set_verify(self.h, int(verify))
        if max_pairs is not None:
            ctx._check(ctx.lib.t3d_server_set_batch_pairs(self.h, int(max_pairs)), "server_set_batch_pairs")

    def close(self):
        if self.h:
            self.ctx.lib.t3d_server_destroy(self.h)
            self.h = None

    def submit(self, j, rid):
        r = abi.Request()
        r.job = j
        r.id = rid
        return self.ctx.lib.t3d_server_submit(self.h, C.byref(r))

    def poll(self, max_n=1024):
        arr = (abi.Completion * max_n)()
        n = C.c_uint32()
        self.ctx.lib.t3d_server_poll(self.h, arr, max_n, C.byref(n))
        return [arr[i] for i in range(n.value)]

    def replay(self, jobs, arrivals):
        n = len(jobs)
        reqs = (abi.Request * n)()
        for i, (j, t) in enumerate(zip(jobs, arrivals)):
            reqs[i].job = j
            reqs[i].id = i
            reqs[i].arrival_s = float(t)
        out = (abi.Completion * n)()
        rc = self.ctx.lib.t3d_server_replay(self.h, reqs, n, out)
        if rc != abi.T3D_OK:
            raise abi.T3DError(rc, "server_replay")
        return [out[i] for i in range(n)]
