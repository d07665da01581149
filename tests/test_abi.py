"""The C ABI without a GPU: every entry point declared in include/t3d.h is
exported by libt3d.so, the ctypes mirror has the header's struct layouts and
constants, and calls fail cleanly (status code, no abort) when no device exists."""
import ctypes as C
import os
import re
import subprocess

import pytest

from tetra3d_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "t3d.h")

STRUCTS = {
    "t3d_material": abi.Material, "t3d_part_desc": abi.PartDesc, "t3d_mesh_desc": abi.MeshDesc,
    "t3d_model_desc": abi.ModelDesc, "t3d_light_desc": abi.LightDesc, "t3d_scene_desc": abi.SceneDesc,
    "t3d_camera_desc": abi.CameraDesc, "t3d_job_desc": abi.JobDesc, "t3d_frame_view": abi.FrameView,
    "t3d_segment_info": abi.SegmentInfo, "t3d_stats": abi.Stats, "t3d_request": abi.Request,
    "t3d_completion": abi.Completion, "t3d_noalloc_args": abi.NoallocArgs, "t3d_raster_opts": abi.RasterOpts,
}


def _header():
    with open(HEADER) as f:
        return f.read()


def _declared_functions():
    text = re.sub(r"/\*.*?\*/", "", _header(), flags=re.S)
    return set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(t3d_[a-z0-9_]+)\s*\(", text, re.M))


def test_header_and_ctypes_mirror_declare_the_same_entry_points():
    assert _declared_functions() == set(abi.SIGNATURES)


def test_library_exports_every_declared_symbol(built):
    lib = abi.load()
    missing = [n for n in _declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if " T " in ln}
    assert _declared_functions() <= exported


def test_struct_layouts_match_the_header(tmp_path):
    """Compiles a C probe against include/t3d.h with gcc and compares every struct's size and
    every field's offset with the ctypes mirror."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "t3d.h"', "int main(void){"]
    for cname, py in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        s, f, v = ln.split()
        got[(s, f)] = int(v)
    for cname, py in STRUCTS.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, f"{cname}.{fname}"


def test_constants_match_the_header():
    defs = dict((m.group(1), int(m.group(2))) for m in re.finditer(r"#define\s+(T3D_[A-Z0-9_]+)\s+(-?\d+)", _header()))
    want = {
        "T3D_OK": abi.T3D_OK, "T3D_E_INVAL": abi.T3D_E_INVAL, "T3D_E_OOM": abi.T3D_E_OOM,
        "T3D_E_ADMIT": abi.T3D_E_ADMIT, "T3D_E_TIMEOUT": abi.T3D_E_TIMEOUT, "T3D_E_CUDA": abi.T3D_E_CUDA,
        "T3D_E_NOTFOUND": abi.T3D_E_NOTFOUND, "T3D_E_BUSY": abi.T3D_E_BUSY,
        "T3D_SORT_BACK_TO_FRONT": abi.SORT_BACK_TO_FRONT, "T3D_SORT_FRONT_TO_BACK": abi.SORT_FRONT_TO_BACK,
        "T3D_SORT_NONE": abi.SORT_NONE, "T3D_TRANSPARENCY_AUTO": abi.TRANSPARENCY_AUTO,
        "T3D_TRANSPARENCY_OPAQUE": abi.TRANSPARENCY_OPAQUE, "T3D_TRANSPARENCY_ALPHA_CLIP": abi.TRANSPARENCY_ALPHA_CLIP,
        "T3D_TRANSPARENCY_TRANSPARENT": abi.TRANSPARENCY_TRANSPARENT, "T3D_MODE_PLAIN": abi.MODE_PLAIN,
        "T3D_MODE_BATCHED": abi.MODE_BATCHED, "T3D_LIGHTING_DEFAULT": abi.LIGHTING_DEFAULT,
        "T3D_LIGHTING_FIXED_NORMALS": abi.LIGHTING_FIXED_NORMALS, "T3D_LIGHTING_DOUBLE_SIDED": abi.LIGHTING_DOUBLE_SIDED,
        "T3D_LV_PER_VERTEX": abi.LV_PER_VERTEX, "T3D_LV_PER_VERTEX_WITH_NORMAL": abi.LV_PER_VERTEX_WITH_NORMAL,
        "T3D_LV_PER_OBJECT": abi.LV_PER_OBJECT, "T3D_LV_OFF": abi.LV_OFF, "T3D_LIGHT_AMBIENT": abi.LIGHT_AMBIENT,
        "T3D_LIGHT_POINT": abi.LIGHT_POINT, "T3D_LIGHT_DIRECTIONAL": abi.LIGHT_DIRECTIONAL,
        "T3D_LIGHT_VOLUME": abi.LIGHT_VOLUME, "T3D_FOG_ADD": abi.FOG_ADD, "T3D_FOG_SUB": abi.FOG_SUB,
        "T3D_FOG_OVERWRITE": abi.FOG_OVERWRITE, "T3D_BILLBOARD_UP_GLOBAL_Y": abi.BILLBOARD_UP_GLOBAL_Y,
        "T3D_BILLBOARD_UP_CAMERA_Y": abi.BILLBOARD_UP_CAMERA_Y, "T3D_DEPTH_DEFAULT": abi.DEPTH_DEFAULT,
        "T3D_DEPTH_UNBILLBOARDED": abi.DEPTH_UNBILLBOARDED,
    }
    for k, v in want.items():
        assert defs.get(k) == v, k


def test_create_without_a_device_returns_a_status(built):
    """No GPU here: t3d_create must return an error code, not abort the process."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = abi.load()
    h = C.c_void_p()
    rc = lib.t3d_create(0, C.byref(h))
    assert rc in (abi.T3D_E_CUDA, abi.T3D_E_INVAL)
    assert not h.value
    # null handles are rejected with a status
    assert lib.t3d_destroy(None) == abi.T3D_E_INVAL
    assert lib.t3d_scene_release(None, 0) == abi.T3D_E_INVAL
    assert lib.t3d_render(None, 0, None, abi.MODE_BATCHED, 0, None) == abi.T3D_E_INVAL


def test_runtime_fails_loudly_without_the_library(tmp_path):
    with pytest.raises(OSError):
        abi.load(str(tmp_path / "missing.so"))
