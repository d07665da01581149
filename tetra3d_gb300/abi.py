"""ctypes mirror of include/t3d.h and the loader for libt3d.so.

The library is the product: every render goes through these C entry points.
load() raises if the CUDA library is missing -- there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libt3d.so")

T3D_OK = 0
T3D_E_INVAL = -1
T3D_E_OOM = -2
T3D_E_ADMIT = -3
T3D_E_TIMEOUT = -4
T3D_E_CUDA = -5
T3D_E_NOTFOUND = -6
T3D_E_BUSY = -7

SORT_BACK_TO_FRONT, SORT_FRONT_TO_BACK, SORT_NONE = 0, 1, 2
TRANSPARENCY_AUTO, TRANSPARENCY_OPAQUE, TRANSPARENCY_ALPHA_CLIP, TRANSPARENCY_TRANSPARENT = 0, 1, 2, 3
LIGHTING_DEFAULT, LIGHTING_FIXED_NORMALS, LIGHTING_DOUBLE_SIDED = 0, 1, 2
LV_PER_VERTEX, LV_PER_VERTEX_WITH_NORMAL, LV_PER_OBJECT, LV_OFF = 0, 1, 2, 3
LIGHT_AMBIENT, LIGHT_POINT, LIGHT_DIRECTIONAL, LIGHT_VOLUME = 0, 1, 2, 3
FOG_ADD, FOG_SUB, FOG_OVERWRITE = 0, 1, 2
BILLBOARD_UP_GLOBAL_Y, BILLBOARD_UP_CAMERA_Y = 0, 1
DEPTH_DEFAULT, DEPTH_UNBILLBOARDED = 0, 1
MODE_PLAIN, MODE_BATCHED = 0, 1

f32p = C.POINTER(C.c_float)
u32p = C.POINTER(C.c_uint32)


class Material(C.Structure):
    _fields_ = [("color", C.c_float * 4), ("tex_w", C.c_float), ("tex_h", C.c_float),
                ("present", C.c_int32), ("backface_culling", C.c_int32), ("sort_mode", C.c_int32),
                ("lighting_mode", C.c_int32), ("lv_shading_mode", C.c_int32), ("shadeless", C.c_int32),
                ("visible", C.c_int32), ("transparency_mode", C.c_int32), ("blend_source_over", C.c_int32),
                ("render_order", C.c_int32), ("billboard", C.c_int32), ("billboard_lock", C.c_int32 * 3),
                ("billboard_up", C.c_int32), ("billboard_depth", C.c_int32), ("texture", C.c_uint32),
                ("texture_filter", C.c_int32), ("texture_map_mode", C.c_int32), ("texture_map_scale", C.c_float * 2),
                ("reserved_tex", C.c_int32)]


class PartDesc(C.Structure):
    _fields_ = [("tri_start", C.c_uint32), ("tri_count", C.c_uint32), ("mat", Material)]


class MeshDesc(C.Structure):
    _fields_ = [("positions", f32p), ("normals", f32p), ("uvs", f32p), ("colors", f32p),
                ("indices", u32p), ("parts", C.POINTER(PartDesc)),
                ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32), ("num_parts", C.c_uint32),
                ("has_dimensions", C.c_int32), ("dim_min", C.c_float * 3), ("dim_max", C.c_float * 3),
                ("shape_positions", f32p), ("shape_normals", f32p), ("shape_weights", f32p),
                ("num_shape_keys", C.c_uint32), ("auto_subdivide", C.c_int32), ("joints", u32p), ("weights", f32p)]


class ModelDesc(C.Structure):
    _fields_ = [("mesh", C.c_uint32), ("visible", C.c_int32), ("frustum_culling", C.c_int32),
                ("shadeless", C.c_int32), ("light_list", C.c_int32), ("use_trs", C.c_int32),
                ("color", C.c_float * 4), ("transform", C.c_float * 16), ("world_rotation", C.c_float * 16),
                ("position", C.c_float * 3), ("scale", C.c_float * 3), ("rotation", C.c_float * 16),
                ("rotate_step", C.c_float * 16), ("skinned", C.c_int32), ("bone_first", C.c_uint32),
                ("batched", C.c_int32), ("batch_owner", C.c_uint32), ("batch_part", C.c_uint32),
                ("reserved", C.c_uint32)]


class LightDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("cell_count", C.c_int32 * 3), ("color", C.c_float * 4),
                ("energy", C.c_float), ("range", C.c_float), ("transform", C.c_float * 16),
                ("world_rotation", C.c_float * 16), ("vol_min", C.c_float * 3), ("vol_max", C.c_float * 3),
                ("cell_size", C.c_float * 3), ("offset", C.c_float * 3), ("bias", C.c_float * 3),
                ("cell_first", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("models", C.POINTER(ModelDesc)),
                ("lights", C.POINTER(LightDesc)), ("volume_cells", f32p),
                ("list_offsets", u32p), ("list_items", u32p),
                ("num_meshes", C.c_uint32), ("num_models", C.c_uint32), ("num_lights", C.c_uint32),
                ("num_volume_cells", C.c_uint32), ("num_lists", C.c_uint32), ("num_bones", C.c_uint32),
                ("bones", f32p), ("subdivision_levels", f32p), ("num_subdivision_levels", C.c_uint32),
                ("max_subdivisions", C.c_uint32), ("cell_use_offsets", u32p), ("cell_use_items", u32p)]


class CameraDesc(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("world_rotation", C.c_float * 16),
                ("width", C.c_int32), ("height", C.c_int32), ("perspective", C.c_int32),
                ("render_depth", C.c_int32), ("perspective_corrected", C.c_int32), ("lighting_on", C.c_int32),
                ("fog_on", C.c_int32), ("fog_mode", C.c_int32), ("fov_y", C.c_float), ("near_plane", C.c_float),
                ("far_plane", C.c_float), ("ortho_scale", C.c_float), ("depth_margin", C.c_float),
                ("fog_range", C.c_float * 2), ("fog_color", C.c_float * 4), ("max_light_count", C.c_int32),
                ("focus_set", C.c_int32), ("focus", C.c_float * 3), ("vertex_snapping", C.c_float)]


class JobDesc(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("reserved", C.c_uint32), ("light_mask", C.c_uint64 * 2),
                ("camera", CameraDesc)]


class FrameView(C.Structure):
    _fields_ = [("xyuv", f32p), ("rgba", f32p), ("depth", f32p), ("seg_base", u32p), ("seg_count", u32p),
                ("num_segments", C.c_uint32), ("reserved", C.c_uint32), ("capacity_tris", C.c_uint64)]


class SegmentInfo(C.Structure):
    _fields_ = [("job", C.c_uint32), ("model", C.c_uint32), ("part", C.c_uint32), ("base", C.c_uint32),
                ("capacity", C.c_uint32), ("count", C.c_uint32), ("draw", C.c_uint32),
                ("draw_transparent", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("visible_tris", C.c_uint64), ("total_tris", C.c_uint64), ("drawn_parts", C.c_uint32),
                ("total_parts", C.c_uint32), ("culled_models", C.c_uint32), ("launches", C.c_uint32),
                ("algorithmic_bytes", C.c_uint64), ("scratch_bytes", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("phase_us", C.c_double * 7), ("phase_busy", C.c_double * 7)]


class Request(C.Structure):
    _fields_ = [("job", JobDesc), ("id", C.c_uint64), ("arrival_s", C.c_double)]


class Completion(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("batch", C.c_uint32),
                ("visible_tris", C.c_uint64), ("arrival_s", C.c_double), ("admit_s", C.c_double),
                ("done_s", C.c_double), ("checksum", C.c_uint64), ("model_bytes", C.c_uint64),
                ("launch_s", C.c_double)]


class NoallocArgs(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p), ("colors", C.c_void_p),
                ("indices", C.c_void_p), ("volume_cells", C.c_void_p), ("out_xyuv", C.c_void_p),
                ("out_rgba", C.c_void_p), ("out_depth", C.c_void_p), ("out_count", C.c_void_p),
                ("model", C.POINTER(ModelDesc)), ("lights", C.POINTER(LightDesc)), ("camera", C.POINTER(CameraDesc)),
                ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32), ("tri_start", C.c_uint32),
                ("tri_count", C.c_uint32), ("num_lights", C.c_uint32), ("reserved", C.c_uint32),
                ("dim_min", C.c_float * 3), ("dim_max", C.c_float * 3), ("mat", Material), ("error", C.c_char * 128)]


class RasterOpts(C.Structure):
    _fields_ = [("fog_curve", C.c_int32), ("dither_size", C.c_float), ("fogless", C.c_int32),
                ("shared_large_tris", C.c_int32)]


class TextureDesc(C.Structure):
    _fields_ = [("rgba8", C.POINTER(C.c_uint8)), ("width", C.c_int32), ("height", C.c_int32)]


# name -> (restype, argtypes) for every entry point of include/t3d.h
_VP = C.c_void_p
SIGNATURES = {
    "t3d_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "t3d_destroy": (C.c_int, [_VP]),
    "t3d_last_error": (C.c_char_p, [_VP]),
    "t3d_set_tuning": (C.c_int, [_VP, C.c_uint32, C.c_uint32, C.c_uint32]),
    "t3d_set_meshlets": (C.c_int, [_VP, C.c_int]),
    "t3d_set_split_phases": (C.c_int, [_VP, C.c_int]),
    "t3d_frame_readback": (C.c_int, [_VP]),
    "t3d_frame_collect": (C.c_int, [_VP, C.POINTER(Stats)]),
    "t3d_set_wait_limit": (C.c_int, [_VP, C.c_uint32]),
    "t3d_scene_upload": (C.c_int, [_VP, C.POINTER(SceneDesc), C.POINTER(C.c_uint32)]),
    "t3d_scene_release": (C.c_int, [_VP, C.c_uint32]),
    "t3d_scene_set_models": (C.c_int, [_VP, C.c_uint32, C.c_uint32, C.POINTER(ModelDesc), C.c_uint32]),
    "t3d_scene_get_transforms": (C.c_int, [_VP, C.c_uint32, f32p, C.c_uint32]),
    "t3d_scene_bytes": (C.c_int, [_VP, C.c_uint32, C.POINTER(C.c_uint64)]),
    "t3d_scene_set_bones": (C.c_int, [_VP, C.c_uint32, C.c_uint32, f32p, C.c_uint32]),
    "t3d_scene_set_lights": (C.c_int, [_VP, C.c_uint32, C.c_uint32, C.POINTER(LightDesc), C.c_uint32]),
    "t3d_scene_set_shape_weights": (C.c_int, [_VP, C.c_uint32, C.c_uint32, f32p, C.c_uint32]),
    "t3d_render": (C.c_int, [_VP, C.c_uint32, C.POINTER(CameraDesc), C.c_int, C.c_int, _VP]),
    "t3d_render_jobs": (C.c_int, [_VP, C.POINTER(JobDesc), C.c_uint32, C.c_int, C.c_int, _VP]),
    "t3d_frame_sync": (C.c_int, [_VP, C.POINTER(Stats)]),
    "t3d_frame_counters": (C.c_int, [_VP, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "t3d_frame_view_get": (C.c_int, [_VP, C.POINTER(FrameView)]),
    "t3d_frame_segments": (C.c_int, [_VP, C.POINTER(SegmentInfo), C.c_uint32, C.POINTER(C.c_uint32)]),
    "t3d_frame_download": (C.c_int, [_VP, f32p, f32p, f32p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "t3d_frame_download_custom0": (C.c_int, [_VP, f32p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "t3d_graph_capture": (C.c_int, [_VP, C.c_uint32, C.POINTER(CameraDesc), C.c_int]),
    "t3d_graph_replay": (C.c_int, [_VP, C.c_uint32, _VP]),
    "t3d_server_create": (C.c_int, [_VP, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(_VP)]),
    "t3d_server_destroy": (C.c_int, [_VP]),
    "t3d_server_set_verify": (C.c_int, [_VP, C.c_int]),
    "t3d_server_set_batch_pairs": (C.c_int, [_VP, C.c_uint32]),
    "t3d_server_submit": (C.c_int, [_VP, C.POINTER(Request)]),
    "t3d_server_poll": (C.c_int, [_VP, C.POINTER(Completion), C.c_uint32, C.POINTER(C.c_uint32)]),
    "t3d_server_replay": (C.c_int, [_VP, C.POINTER(Request), C.c_uint32, C.POINTER(Completion)]),
    "t3d_render_part_noalloc": (C.c_int, [C.c_int, C.POINTER(NoallocArgs), _VP]),
    "t3d_frame_raster": (C.c_int, [_VP, C.c_uint32, C.POINTER(RasterOpts), _VP]),
    "t3d_raster_set_textures": (C.c_int, [_VP, C.POINTER(TextureDesc), C.c_uint32]),
    "t3d_frame_images": (C.c_int, [_VP, C.POINTER(C.c_uint8), C.POINTER(C.c_uint8), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32)]),
}

_lib = None


def load(path=LIB_PATH):
    """Loads libt3d.so (raises OSError if it was not built)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"libt3d.so not built at {path}: run __graft_entry__.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


class T3DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"t3d error {code}: {msg}")
        self.code = code


def fptr(a):
    return a.ctypes.data_as(f32p) if a is not None else None


def uptr(a):
    return a.ctypes.data_as(u32p) if a is not None else None


def mat_array(m):
    """numpy (4,4) or (16,) float32 -> ctypes float[16]."""
    a = np.ascontiguousarray(np.asarray(m, dtype=np.float32).reshape(16))
    return (C.c_float * 16)(*a.tolist())
