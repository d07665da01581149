"""Generates tests/golden/c1_whole_path.npz: the emitted stream of the one-sphere scene
(a UV sphere of 32 x 16 segments, 960 triangles, ambient + directional + point light,
640x360, back-to-front sort), of the same scene with a non-uniform scale and two more
point lights, and of that scene with a light volume (a grid of cells, an offset and a light
bias) lighting the sphere per vertex, per vertex with the normal, and per object, with fog,
with fixed-normal and double-sided lighting, without backface culling, front-to-back and
unsorted, lit by a LightGroup, and seen with perspective-corrected texture mapping, vertex
snapping or lighting off, or through an orthographic camera, and a frame of six such
models (two outside the frustum, three lit by a LightGroup), computed by
a second restatement of the vertex stage written here in numpy binary32 arithmetic,
independently of the C++ oracle, so the oracle can be checked against it bit for bit.

Every operation is an elementwise IEEE binary32 operation (numpy float32 arrays, no
fused multiply-add, no reductions), in the order the reference writes it:

- Node.Transform (node.go:572-607), Matrix4.Mult (matrix_none.go:6-32; the amd64
  assembly in matrix_amd64.s sums in the same order), Inverted (matrix.go:255-307),
  Decompose (matrix.go:181-196), MultVec / MultVecW (matrix.go:619-637), the
  projection and view matrices (matrix.go:588-607, camera.go:638-679);
- Camera.SphereInFrustum (camera.go:933-984) for the model's culling sphere
  (model.go:394-395, colliderSphere.go:51-58);
- Model.ProcessVertices (model.go:600-995): MVP, near/far, the +-0.5 screen test,
  2D backface test, the model-space camera distance to Triangle.Center
  (mesh.go:1972-1982) as the depth key;
- sortingTriangleBucket.Sort / ForEach (sortingTriangles.go:38-125), 512 bins;
- lights: AmbientLight, PointLight, DirectionalLight beginRender / beginModel /
  VertexLight (light.go:110-360) with the model-level point-light range skip
  (camera.go:1613-1641); LightVolume.VertexLight (light.go:583-663) with the cell grid of
  LightVolumeResize (light.go:459-513), convertToXYZIndices (light.go:716-724) and
  Dimensions.Contains (mesh.go:82-84);
- the emit loop (camera.go:1646-1820): screen position, UV, colour x lighting, depth, and
  the world's fog added to or multiplied into the colour when the depth is not rendered
  (camera.go:1785-1812).

Run from the repo root: python tests/golden/make_c1_whole_path.py
"""
import hashlib
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

F = np.float32
BINS = 512


# ---- Matrix4 (row-major 4x4 float32; m[r][c]) ----

def ident():
    return np.eye(4, dtype=F)


def mmul(a, b):
    """Matrix4.Mult: out[i][j] = ((a[i][0]*b[0][j] + a[i][1]*b[1][j]) + a[i][2]*b[2][j]) + a[i][3]*b[3][j]."""
    a = a.astype(F)
    b = b.astype(F)
    return ((a[:, 0:1] * b[0:1, :] + a[:, 1:2] * b[1:2, :]) + a[:, 2:3] * b[2:3, :]) + a[:, 3:4] * b[3:4, :]


def translate(x, y, z):
    m = ident()
    m[3, 0], m[3, 1], m[3, 2] = x, y, z
    return m


def scale(x, y, z):
    m = ident()
    m[0, 0], m[1, 1], m[2, 2] = x, y, z
    return m


def transposed(m):
    return np.ascontiguousarray(m.T)


def inverted(m):
    """Matrix4.Inverted: 2x2 minors of the lower rows, cofactor expansion, one reciprocal."""
    m = m.astype(F)
    g = lambda r, c: m[r, c]
    A2323 = g(2, 2) * g(3, 3) - g(2, 3) * g(3, 2)
    A1323 = g(2, 1) * g(3, 3) - g(2, 3) * g(3, 1)
    A1223 = g(2, 1) * g(3, 2) - g(2, 2) * g(3, 1)
    A0323 = g(2, 0) * g(3, 3) - g(2, 3) * g(3, 0)
    A0223 = g(2, 0) * g(3, 2) - g(2, 2) * g(3, 0)
    A0123 = g(2, 0) * g(3, 1) - g(2, 1) * g(3, 0)
    A2313 = g(1, 2) * g(3, 3) - g(1, 3) * g(3, 2)
    A1313 = g(1, 1) * g(3, 3) - g(1, 3) * g(3, 1)
    A1213 = g(1, 1) * g(3, 2) - g(1, 2) * g(3, 1)
    A2312 = g(1, 2) * g(2, 3) - g(1, 3) * g(2, 2)
    A1312 = g(1, 1) * g(2, 3) - g(1, 3) * g(2, 1)
    A1212 = g(1, 1) * g(2, 2) - g(1, 2) * g(2, 1)
    A0313 = g(1, 0) * g(3, 3) - g(1, 3) * g(3, 0)
    A0213 = g(1, 0) * g(3, 2) - g(1, 2) * g(3, 0)
    A0312 = g(1, 0) * g(2, 3) - g(1, 3) * g(2, 0)
    A0212 = g(1, 0) * g(2, 2) - g(1, 2) * g(2, 0)
    A0113 = g(1, 0) * g(3, 1) - g(1, 1) * g(3, 0)
    A0112 = g(1, 0) * g(2, 1) - g(1, 1) * g(2, 0)
    det = (((g(0, 0) * ((g(1, 1) * A2323 - g(1, 2) * A1323) + g(1, 3) * A1223)
             - g(0, 1) * ((g(1, 0) * A2323 - g(1, 2) * A0323) + g(1, 3) * A0223))
            + g(0, 2) * ((g(1, 0) * A1323 - g(1, 1) * A0323) + g(1, 3) * A0123))
           - g(0, 3) * ((g(1, 0) * A1223 - g(1, 1) * A0223) + g(1, 2) * A0123))
    det = F(1) / det

    def c3(a, x, b, y, c, z):  # (a*x - b*y) + c*z, left to right
        return (a * x - b * y) + c * z

    o = ident()
    o[0, 0] = det * c3(g(1, 1), A2323, g(1, 2), A1323, g(1, 3), A1223)
    o[0, 1] = det * -c3(g(0, 1), A2323, g(0, 2), A1323, g(0, 3), A1223)
    o[0, 2] = det * c3(g(0, 1), A2313, g(0, 2), A1313, g(0, 3), A1213)
    o[0, 3] = det * -c3(g(0, 1), A2312, g(0, 2), A1312, g(0, 3), A1212)
    o[1, 0] = det * -c3(g(1, 0), A2323, g(1, 2), A0323, g(1, 3), A0223)
    o[1, 1] = det * c3(g(0, 0), A2323, g(0, 2), A0323, g(0, 3), A0223)
    o[1, 2] = det * -c3(g(0, 0), A2313, g(0, 2), A0313, g(0, 3), A0213)
    o[1, 3] = det * c3(g(0, 0), A2312, g(0, 2), A0312, g(0, 3), A0212)
    o[2, 0] = det * c3(g(1, 0), A1323, g(1, 1), A0323, g(1, 3), A0123)
    o[2, 1] = det * -c3(g(0, 0), A1323, g(0, 1), A0323, g(0, 3), A0123)
    o[2, 2] = det * c3(g(0, 0), A1313, g(0, 1), A0313, g(0, 3), A0113)
    o[2, 3] = det * -c3(g(0, 0), A1312, g(0, 1), A0312, g(0, 3), A0112)
    o[3, 0] = det * -c3(g(1, 0), A1223, g(1, 1), A0223, g(1, 2), A0123)
    o[3, 1] = det * c3(g(0, 0), A1223, g(0, 1), A0223, g(0, 2), A0123)
    o[3, 2] = det * -c3(g(0, 0), A1213, g(0, 1), A0213, g(0, 2), A0113)
    o[3, 3] = det * c3(g(0, 0), A1212, g(0, 1), A0212, g(0, 2), A0112)
    return o


def sqrt32(x):
    """math32.Sqrt: the float64 square root rounded to float32 (the correctly rounded float32 root)."""
    return F(math.sqrt(float(x)))


def mag3(x, y, z):
    return sqrt32((x * x + y * y) + z * z)


def unit3(v):
    """Vector3.Unit / Vector4.Unit (xyz only): unchanged when the length is < 1e-8 or exactly 1."""
    x, y, z = F(v[0]), F(v[1]), F(v[2])
    l = mag3(x, y, z)
    if l < F(1e-8) or l == F(1):
        return [x, y, z]
    return [x / l, y / l, z / l]


def decompose(m):
    """Matrix4.Decompose: position = row 3, rotation rows = unit rows 0-2 (w kept), scale = row lengths
    of m x rotation^T."""
    pos = [m[3, 0], m[3, 1], m[3, 2]]
    rot = ident()
    for r in range(3):
        ux, uy, uz = unit3(m[r, :3])
        rot[r, 0], rot[r, 1], rot[r, 2], rot[r, 3] = ux, uy, uz, m[r, 3]
    inn = mmul(m, transposed(rot))
    scl = [mag3(inn[r, 0], inn[r, 1], inn[r, 2]) for r in range(3)]
    return pos, scl, rot


def multvec(m, v):
    """MultVec: x' = ((m00 x + m10 y) + m20 z) + m30 (v may be arrays)."""
    x, y, z = v
    return [((m[0, c] * x + m[1, c] * y) + m[2, c] * z) + m[3, c] for c in range(3)]


def multvecw(m, v):
    x, y, z = v
    return [((m[0, c] * x + m[1, c] * y) + m[2, c] * z) + m[3, c] for c in range(4)]


def node_transform(pos, scl, rot):
    """Node.Transform for a node without parent: Scale x Rotation x Translate."""
    t = mmul(scale(*scl), rot)
    return mmul(t, translate(*pos))


def projection(fov, near, far, w, h):
    """NewProjectionMatrix4Perspective; math32.Tan is the float64 tangent rounded to float32."""
    aspect = F(w) / F(h)
    t = F(math.tan(float((F(fov) * F(math.pi)) / F(360))))
    b = -t
    r = t * aspect
    l = -r
    near, far = F(near), F(far)
    P = np.zeros((4, 4), F)
    P[0, 0] = (F(2) * near) / (r - l)
    P[0, 2] = (r + l) / (r - l)
    P[1, 1] = (F(2) * near) / (t - b)
    P[1, 2] = (t + b) / (t - b)
    P[2, 2] = -((far + near) / (far - near))
    P[2, 3] = -(((F(2) * far) * near) / (far - near))
    P[3, 2] = F(-1)
    return P


def projection_ortho(near, far, w, h, scale):
    """Camera.Projection for an orthographic camera (camera.go:669-675): NewProjectionMatrix4Orthographic
    (matrix.go:609-616) with right / left = +-orthoScale and top / bottom = +-(h / w) * orthoScale."""
    asr = F(h) / F(w)
    right, left = F(1) * scale, F(-1) * scale
    top, bottom = asr * scale, -asr * scale
    near, far = F(near), F(far)
    P = np.zeros((4, 4), F)
    P[0, 0] = F(2) / (right - left)
    P[1, 1] = F(2) / (top - bottom)
    P[2, 2] = F(-2) / (far - near)
    P[3, 3] = F(1)
    return P


# ---- the scene ----

def scene_inputs(sd, model=0, part=0):
    """The binary32 inputs the restatement reads from a SceneData for one render pair: a model and
    one part of its mesh (the part's triangles and material; the mesh's vertices and
    dimensions)."""
    from tetra3d_gb300 import abi
    assert 0 <= model < sd.nmodels
    mv = sd.mv[model]
    me = sd.meshes[int(mv["mesh"])]
    mat = me.parts[part]["mat"]
    t0, nt = int(me.parts[part]["tri_start"]), int(me.parts[part]["tri_count"])
    cam = sd.camera
    def light_dict(L):
        Lt = np.asarray(L.transform[:], F).reshape(4, 4)
        return dict(type=int(L.type), color=np.asarray(L.color[:3], F), energy=F(L.energy),
                           range=F(L.range), world_pos=[Lt[3, 0], Lt[3, 1], Lt[3, 2]],
                           world_rot=np.asarray(L.world_rotation[:], F).reshape(4, 4),
                           vol_min=np.asarray(L.vol_min[:], F), vol_max=np.asarray(L.vol_max[:], F),
                           cell_size=np.asarray(L.cell_size[:], F), offset=np.asarray(L.offset[:], F),
                           bias=np.asarray(L.bias[:], F), cell_count=[int(c) for c in L.cell_count],
                           cell_first=int(L.cell_first))
    ll = int(mv["light_list"])  # -1: the scene's light list (list 0); k >= 1: LightGroup k
    lights = [light_dict(sd.lights[k]) for k in sd.lists[ll if ll >= 0 else 0]]
    all_lights = [light_dict(sd.lights[k]) for k in range(sd.nlights)]
    cell_uses = None if sd.cell_uses is None else [list(map(int, u)) for u in sd.cell_uses]
    ct = np.asarray(cam.transform[:], F).reshape(4, 4)
    return dict(
        positions=me.positions.astype(F), normals=me.normals.astype(F), uvs=me.uvs.astype(F),
        colors=None if me.colors is None else me.colors.astype(F), indices=np.asarray(me.indices, np.int64).reshape(-1, 3)[t0:t0 + nt], tri_base=t0,
        model_pos=np.asarray(mv["position"], F), model_scale=np.asarray(mv["scale"], F),
        model_rot=np.asarray(mv["rotation"], F).reshape(4, 4), model_color=np.asarray(mv["color"], F),
        mat_color=np.asarray(mat["color"], F), tex=(F(mat["tex_w"]), F(mat["tex_h"])),
        backface=bool(mat["backface_culling"]), sort_mode=int(mat["sort_mode"]),
        lighting_mode=int(mat["lighting_mode"]), shadeless=bool(mat["shadeless"]) or bool(mv["shadeless"]),
        lv_mode=int(mat["lv_shading_mode"]), cells=np.asarray(sd.cells, F)[:max(0, sd.ncells)],
        all_lights=all_lights, cell_uses=cell_uses,
        lights=lights, cam_pos=[ct[3, 0], ct[3, 1], ct[3, 2]],
        cam_rot=np.asarray(cam.world_rotation[:], F).reshape(4, 4), width=int(cam.width), height=int(cam.height),
        fov=F(cam.fov_y), near=F(cam.near_plane), far=F(cam.far_plane), depth_margin=F(cam.depth_margin),
        perspective=bool(cam.perspective), lighting_on=bool(cam.lighting_on), render_depth=bool(cam.render_depth),
        fog_on=bool(cam.fog_on), fog_mode=int(cam.fog_mode), fog_range=np.asarray(cam.fog_range[:], F),
        fog_color=np.asarray(cam.fog_color[:3], F), pcorrect=bool(cam.perspective_corrected),
        snap=F(cam.vertex_snapping), ortho_scale=F(cam.ortho_scale),
        skinned=bool(mv["skinned"]), bone_first=int(mv["bone_first"]),
        joints=None if me.joints is None else np.asarray(me.joints, np.int64),
        weights=None if me.weights is None else np.asarray(me.weights, F),
        bones=None if not bool(mv["skinned"]) else np.asarray(sd.bones, F).reshape(-1, 4, 4),
        shape_positions=None if me.shape_weights is None else np.asarray(me.shape_positions, F),
        shape_normals=None if me.shape_weights is None else np.asarray(me.shape_normals, F),
        shape_weights=None if me.shape_weights is None else np.asarray(me.shape_weights, F),
        abi=abi)


def in_frustum(S, M, dmin, dmax, skinned=False):
    """Camera.SphereInFrustum for the model's culling sphere as Model.onTransformUpdate places it
    (model.go:141-181): position + (rotation x Dimensions.Center()) * scale, radius = MaxSpan of the
    scaled Dimensions / 2; the sphere node itself is unscaled (colliderSphere.go:51-60)."""
    pos, scl, rot = decompose(M)
    # a skinned model's sphere sits on the model position: its centre stays the zero vector
    centre = [F(0)] * 3 if skinned else [(dmax[a] + dmin[a]) / F(2) for a in range(3)]
    cr = multvec(rot, centre)
    wpos = [pos[a] + cr[a] * scl[a] for a in range(3)]
    lo = [dmin[a] * scl[a] for a in range(3)]
    hi = [dmax[a] * scl[a] for a in range(3)]
    radius = mag3(hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]) / F(2)
    crot = S["cam_rot"]
    fwd, right, up = unit3(crot[2, :3]), unit3(crot[0, :3]), unit3(crot[1, :3])
    diff = [wpos[a] - S["cam_pos"][a] for a in range(3)]
    dot = lambda a, b: (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]
    pcz = dot(diff, [-fwd[0], -fwd[1], -fwd[2]])
    if pcz > S["far"] + radius or pcz < S["near"] - radius:
        return False
    if not S["perspective"]:  # the orthographic box (camera.go:963-979)
        width = S["ortho_scale"]
        height = width / (F(S["width"]) / F(S["height"]))
        pcy = dot(diff, up)
        if -height / F(2) - radius > pcy or pcy > height / F(2) + radius:
            return False
        pcx = dot(diff, right)
        return not (-width / F(2) - radius > pcx or pcx > width / F(2) + radius)
    angle = (S["fov"] * F(3.1415)) / F(360)
    tang = F(math.tan(float(angle)))
    fy = F(1) / F(math.cos(float(angle)))
    aspect = F(S["width"]) / F(S["height"])
    fx = F(1) / F(math.cos(float(F(math.atan(float(tang * aspect))))))
    d = fy * radius
    pcz = pcz * tang
    pcy = dot(diff, up)
    if pcy > pcz + d or pcy < -pcz - d:
        return False
    pcz = pcz * aspect
    d = fx * radius
    pcx = dot(diff, right)
    return not (pcx > pcz + d or pcx < -pcz - d)


def keyed_vertices(S):
    """Mesh.VertexPositionWithShapeKeys / VertexNormalWithShapeKeys (mesh.go:796-822): each shape
    key, in order, adds its delta times its weight to the base position and normal."""
    P, N = S["positions"].copy(), S["normals"].copy()
    if S["shape_weights"] is not None:
        for k, w in enumerate(S["shape_weights"]):
            P = (P + S["shape_positions"][k] * w).astype(F)
            N = (N + S["shape_normals"][k] * w).astype(F)
    return P, N


def skin_vertices(S, P, N):
    """Model.skinVertex (model.go:559-594) for every vertex: the skin matrix starts at zero, each
    non-zero weight adds the bone influence scaled by it element by element (Matrix4.Add / Scale,
    matrix.go:639-661), and a weight of exactly 1 replaces the sum and ends the loop; the (keyed)
    position goes through the matrix, the normal through it with its last row set to (0, 0, 0, 1)."""
    J, Wt, B = S["joints"], S["weights"], S["bones"]
    nv = len(P)
    m = np.zeros((nv, 4, 4), F)
    done = np.zeros(nv, bool)
    for k in range(4):
        w = Wt[:, k]
        bone = B[S["bone_first"] + J[:, k]]
        one = ~done & (w == F(1))
        add = ~done & (w != F(0)) & ~one
        m = np.where(add[:, None, None], (m + bone * w[:, None, None]).astype(F), m)
        m = np.where(one[:, None, None], bone, m)
        done |= one
    pos = [((P[:, 0] * m[:, 0, c] + P[:, 1] * m[:, 1, c]) + P[:, 2] * m[:, 2, c]) + m[:, 3, c] for c in range(3)]
    mn = m.copy()
    mn[:, 3, :] = np.array([0, 0, 0, 1], F)
    nrm = [((N[:, 0] * mn[:, 0, c] + N[:, 1] * mn[:, 1, c]) + N[:, 2] * mn[:, 2, c]) + mn[:, 3, c] for c in range(3)]
    return np.stack(pos, 1).astype(F), np.stack(nrm, 1).astype(F)


def grid_counts(vmin, vmax, cs):
    """LightVolumeResize (light.go:485-513): cells along an axis from Min + size/2, stepping by the
    size in binary32 while the position stays <= Max - size/2."""
    out = []
    for a in range(3):
        n = 0
        v = F(vmin[a]) + F(cs[a] / F(2))
        top = F(vmax[a]) - F(cs[a] / F(2))
        while v <= top:
            n += 1
            v = F(v + cs[a])
        out.append(n)
    return out


def round_half_away(x):
    """math32.Round: float32(math.Round(float64(x))), halves away from zero."""
    x = np.asarray(x, np.float64)
    return np.where(x < 0, -np.floor(-x + 0.5), np.floor(x + 0.5))


def volume_cells(S, L, M, P, N):
    """LightVolume.VertexLight (light.go:583-663) for every vertex of an unskinned model: the cell
    colour each vertex takes (black where no cell), whether the vertex adds anything (the light
    returns early for vertices outside the volume's dimensions) and the scene cell whose
    useLights light it first (-1: none)."""
    abi = S["abi"]
    mode = S["lv_mode"]
    nv = len(P)
    if mode == abi.LV_OFF:  # LightVolume.Light skips the pair
        z = np.zeros(nv, F)
        return z, z, z, np.zeros(nv, bool), np.full(nv, -1)
    vmin, vmax, cs, off, bias = L["vol_min"], L["vol_max"], L["cell_size"], L["offset"], L["bias"]
    cnt = grid_counts(vmin, vmax, cs)
    assert cnt == L["cell_count"], (cnt, L["cell_count"])
    cells = S["cells"]

    def cell_rgb(wx, wy, wz):
        # convertToXYZIndices: int(Round(((w - offset - Min - size/2) / size)))
        idx = []
        for a, w in enumerate((wx, wy, wz)):
            q = (((np.asarray(w, F) - off[a]) - vmin[a]) - (cs[a] / F(2))) / cs[a]
            idx.append(round_half_away(q.astype(F)).astype(np.int64))
        x, y, z = idx
        inside = (x >= 0) & (y >= 0) & (z >= 0) & (x < cnt[0]) & (y < cnt[1]) & (z < cnt[2])
        flat = np.where(inside, x + y * cnt[0] + z * cnt[0] * cnt[1], 0)
        rgb = cells[L["cell_first"] + flat, :3].astype(F)
        rgb = np.where(inside[..., None], rgb, F(0)).astype(F)
        return rgb[..., 0], rgb[..., 1], rgb[..., 2], np.where(inside, L["cell_first"] + flat, -1)

    if mode == abi.LV_PER_OBJECT:  # the cell at Model.WorldPosition, for every vertex (no useLights)
        r, g, b, _ = cell_rgb(np.full(nv, M[3, 0], F), np.full(nv, M[3, 1], F), np.full(nv, M[3, 2], F))
        return r, g, b, np.ones(nv, bool), np.full(nv, -1)
    half = [cs[a] / F(2) for a in range(3)]
    if mode == abi.LV_PER_VERTEX_WITH_NORMAL:
        # only vertPosWithNormal is set in this mode: the containment test reads vertPos, which
        # stays the zero vector
        q = [P[:, a] + N[:, a] * half[a] for a in range(3)]
        t = multvec(M, (q[0], q[1], q[2]))
        look = [t[a] + bias[a] for a in range(3)]
        probe = [np.zeros(nv, F)] * 3
    else:
        t = multvec(M, (P[:, 0], P[:, 1], P[:, 2]))
        look = probe = [t[a] + bias[a] for a in range(3)]
    contains = ((probe[0] >= vmin[0]) & (probe[1] >= vmin[1]) & (probe[2] >= vmin[2]) &
                (probe[0] <= vmax[0]) & (probe[1] <= vmax[1]) & (probe[2] <= vmax[2]))
    r, g, b, cell = cell_rgb(*look)
    return r, g, b, contains, np.where(contains, cell, -1)


def render(S, want_custom0=False):
    """The vertex stage for the scene's one model and one mesh part: returns (triangle order, xyuv,
    rgba, depth) of the visible triangles in draw order, and Custom0 (1 / w per corner under
    perspective-corrected texture mapping, else None) when want_custom0."""
    abi = S["abi"]
    P, N, UV, idx = S["positions"], S["normals"], S["uvs"], S["indices"]
    W, H = S["width"], S["height"]
    near, far = S["near"], S["far"]
    # camera: view = T(-pos) x R^T, vp = view x projection (camera.go:638-648, :1329)
    cp = S["cam_pos"]
    view = mmul(translate(-cp[0], -cp[1], -cp[2]), transposed(S["cam_rot"]))
    if S["perspective"]:
        vp = mmul(view, projection(S["fov"], near, far, W, H))
    else:
        vp = mmul(view, projection_ortho(near, far, W, H, S["ortho_scale"]))
    # model transform and the culling sphere
    M = node_transform(S["model_pos"], S["model_scale"], S["model_rot"])
    dmin = [F(P[:, a].min()) for a in range(3)]  # Mesh.UpdateDimensions
    dmax = [F(P[:, a].max()) for a in range(3)]
    maxspan = mag3(dmax[0] - dmin[0], dmax[1] - dmin[1], dmax[2] - dmin[2])
    skinned = S["skinned"]
    # shape keys move the vertices; the dimensions and the triangle centres stay on the base mesh
    Pk, Nk = keyed_vertices(S)
    if not in_frustum(S, M, dmin, dmax, skinned):
        return np.zeros(0, np.int64), np.zeros((0, 3, 4), F), np.zeros((0, 3, 4), F), np.zeros((0, 3), F)
    # ProcessVertices
    mvp = mmul(M, vp)
    ip, isc, ir = decompose(inverted(M))
    rc = multvec(ir, cp)
    icam = [rc[a] + ip[a] * (F(1) / isc[a]) for a in range(3)]
    if skinned:  # world-space vertices through the skin, then VP alone (model.go:755-770)
        Pw, Nw = skin_vertices(S, Pk, Nk)
        clip = multvecw(vp, (Pw[:, 0], Pw[:, 1], Pw[:, 2]))
    else:
        clip = multvecw(mvp, (Pk[:, 0], Pk[:, 1], Pk[:, 2]))  # per vertex, float32 arrays
    X, Y, Z, Wc = clip
    if S["snap"] > F(0):  # Camera.VertexSnapping (model.go:813-818): math32.Round = half away from zero
        sn = S["snap"]
        X = (round_half_away(X * sn).astype(F) / sn).astype(F)
        Y = (round_half_away(Y * sn).astype(F) / sn).astype(F)
        Z = (round_half_away(Z * sn).astype(F) / sn).astype(F)
    a, b, c = idx[:, 0], idx[:, 1], idx[:, 2]
    inb = np.zeros(len(idx), bool)
    for k in (a, b, c):
        inb |= (Z[k] + F(1) >= near) & (Z[k] < far)
    wq = np.where(Wc < 0, F(0.000001), Wc).astype(F)
    sx, sy = X / wq, Y / wq
    vis = inb.copy()
    for comp in (sx, sy):
        vis &= ~((comp[a] < F(-0.5)) & (comp[b] < F(-0.5)) & (comp[c] < F(-0.5)))
        vis &= ~((comp[a] > F(0.5)) & (comp[b] > F(0.5)) & (comp[c] > F(0.5)))
    if S["backface"]:
        n0x, n0y = sx[a] - sx[b], sy[a] - sy[b]
        n1x, n1y = sx[b] - sx[c], sy[b] - sy[c]
        vis &= ~((n0x * n1y) - (n1x * n0y) < F(0))
    if skinned:  # the skinned centre, summed from zero, against the world camera (model.go:839-863, :941-946)
        ctr = [(((F(0) + Pw[a, k]) + Pw[b, k]) + Pw[c, k]) / F(3) for k in range(3)]
        dx, dy, dz = cp[0] - ctr[0], cp[1] - ctr[1], cp[2] - ctr[2]
    else:
        ctr = [((P[a, k] + P[b, k]) + P[c, k]) / F(3) for k in range(3)]  # Triangle.RecalculateCenter
        dx, dy, dz = icam[0] - ctr[0], icam[1] - ctr[1], icam[2] - ctr[2]
    depth = (dx * dx + dy * dy) + dz * dz
    vis &= np.isfinite(depth)
    tris = np.nonzero(vis)[0]
    # sortingTriangleBucket.Sort: bins of the accepted triangles, in triangle order within a bin
    if len(tris):
        mn, mx = F(depth[tris].min()), F(depth[tris].max())
    else:
        mn, mx = F(np.finfo(F).max), -F(np.finfo(F).max)
    rng = mx - mn
    if rng == F(0):
        rng = rng + F(0.001)
    if S["sort_mode"] != abi.SORT_NONE:
        key = ((depth[tris] - mn) / rng) * F(BINS)
        t = np.where(key < F(0), F(0), np.where(key > F(BINS - 1), F(BINS - 1), key))
        bins = t.astype(np.int64)
    else:
        bins = np.zeros(len(tris), np.int64)
    walk = (BINS - 1 - bins) if S["sort_mode"] == abi.SORT_BACK_TO_FRONT else bins
    order = tris[np.argsort(walk, kind="stable")]
    # lighting (camera.go:1521-1641; light.go:110-360), a sum over the model's lights in list order
    lighting = S["lighting_on"] and not S["shadeless"]
    nv = len(P)
    lr = np.zeros(nv, F)
    lg = np.zeros(nv, F)
    lb = np.zeros(nv, F)
    if lighting:
        mpos = [M[3, 0], M[3, 1], M[3, 2]]  # Model.WorldPosition
        mrot_inv_t = transposed(inverted(S["model_rot"]))  # DirectionalLight.beginModel
        if skinned:  # the lights work on the skinned world-space vertices (light.go:183-186, :334-343)
            vx, vy, vz = Pw[:, 0], Pw[:, 1], Pw[:, 2]
            nx, ny, nz = Nw[:, 0], Nw[:, 1], Nw[:, 2]
        else:
            vx, vy, vz = Pk[:, 0], Pk[:, 1], Pk[:, 2]
            nx, ny, nz = Nk[:, 0], Nk[:, 1], Nk[:, 2]
        def add(lr, lg, lb, on, tr, tg, tb):
            return (np.where(on, lr + tr, lr).astype(F), np.where(on, lg + tg, lg).astype(F),
                    np.where(on, lb + tb, lb).astype(F))

        def light_one(L, lr, lg, lb, mask, nested):
            """One light's VertexLight on the vertices of `mask` (a cell's useLights when nested:
            no model-level range skip, camera.go:1625-1629 applies to the scene's lights)."""
            col, e = L["color"], L["energy"]
            if L["type"] == abi.LIGHT_AMBIENT:
                res = [col[0] * e, col[1] * e, col[2] * e]  # beginRender
                return add(lr, lg, lb, mask, res[0], res[1], res[2])
            if L["type"] == abi.LIGHT_DIRECTIONAL:
                fwd = unit3(L["world_rot"][2, :3])  # WorldRotation().Forward()
                if S["lighting_mode"] == abi.LIGHTING_FIXED_NORMALS:
                    wn = [np.full(nv, fwd[0], F), np.full(nv, fwd[1], F), np.full(nv, fwd[2], F)]
                elif skinned:
                    wn = [nx, ny, nz]
                else:
                    wn = multvec(mrot_inv_t, (nx, ny, nz))
                df = (wn[0] * fwd[0] + wn[1] * fwd[1]) + wn[2] * fwd[2]
                if S["lighting_mode"] == abi.LIGHTING_DOUBLE_SIDED:
                    df = np.abs(df)
                return add(lr, lg, lb, mask & (df > F(0)), (col[0] * df) * e, (col[1] * df) * e, (col[2] * df) * e)
            if L["type"] == abi.LIGHT_POINT:
                R = L["range"]
                R2 = R * R
                lp = L["world_pos"]
                if R > F(0) and not nested:  # model-level skip (camera.go:1625-1629)
                    dist = maxspan + R
                    ddx, ddy, ddz = mpos[0] - lp[0], mpos[1] - lp[1], mpos[2] - lp[2]
                    if (ddx * ddx + ddy * ddy) + ddz * ddz > dist * dist:
                        return lr, lg, lb
                if skinned:  # PointLight.beginModel: the light's own world position
                    wp = [F(lp[0]), F(lp[1]), F(lp[2])]
                else:
                    p_, s_, r_ = decompose(inverted(M))  # PointLight.beginModel
                    rq = multvec(r_, lp)
                    wp = [rq[k] + p_[k] * (F(1) / s_[k]) for k in range(3)]
                ex, ey, ez = wp[0] - vx, wp[1] - vy, wp[2] - vz
                dist2 = (ex * ex + ey * ey) + ez * ez
                with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                    if R > F(0):
                        on = ~(dist2 > R2)
                    else:
                        on = ~((F(1) / dist2) * e < F(0.001))
                    l = np.sqrt(((ex * ex + ey * ey) + ez * ez).astype(np.float64)).astype(F)
                    keep = (l < F(1e-8)) | (l == F(1))
                    ux = np.where(keep, ex, ex / l).astype(F)
                    uy = np.where(keep, ey, ey / l).astype(F)
                    uz = np.where(keep, ez, ez / l).astype(F)
                if S["lighting_mode"] == abi.LIGHTING_FIXED_NORMALS:
                    qx, qy, qz = ux, uy, uz
                else:
                    qx, qy, qz = nx, ny, nz
                dif = (qx * ux + qy * uy) + qz * uz
                if S["lighting_mode"] == abi.LIGHTING_DOUBLE_SIDED:
                    dif = np.abs(dif)
                on &= dif > F(0)
                with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                    dfac = (dif * (F(1) / (F(1) + (F(0.1) * dist2)))) * F(2)
                    if R2 > F(0):
                        q = (R2 - dist2) / dist2
                        q = np.where(q < F(0), F(0), np.where(q > F(1), F(1), q)).astype(F)
                        dfac = dfac * q
                return add(lr, lg, lb, mask & on, (col[0] * dfac) * e, (col[1] * dfac) * e, (col[2] * dfac) * e)
            if L["type"] == abi.LIGHT_VOLUME:
                cr_, cg_, cb_, on, cell = volume_cells(S, L, M, Pk, Nk)
                on &= mask
                # the cell's useLights first, in list order, on the vertices in that cell (light.go:650-656)
                if S["cell_uses"] is not None and not nested:
                    for c in sorted(set(cell[on & (cell >= 0)].tolist())):
                        for u in S["cell_uses"][c]:
                            lr, lg, lb = light_one(S["all_lights"][u], lr, lg, lb, on & (cell == c), True)
                return add(lr, lg, lb, on, (col[0] * cr_) * e, (col[1] * cg_) * e, (col[2] * cb_) * e)
            return lr, lg, lb

        every = np.ones(nv, bool)
        for L in S["lights"]:
            lr, lg, lb = light_one(L, lr, lg, lb, every, False)
    # the emit loop, corner by corner in draw order
    mp = S["model_color"] * S["mat_color"]  # Color4.MultiplyRGBA
    margin = (far - near) * S["depth_margin"]
    spread = (far - near) + (margin * F(2))
    tw, th = S["tex"]
    cor = idx[order]  # (n, 3) vertex per corner
    w = Wc[cor] if S["perspective"] else np.ones(cor.shape, F)
    w = np.where(w < F(0), F(0.001), w).astype(F)
    xs = (X[cor] / w) * F(W) + F(W) / F(2)
    ys = (Y[cor] / -w) * F(H) + F(H) / F(2)
    if S["pcorrect"]:  # camera.go:1689-1704: UV over w, and Custom0 = 1 / w
        u = (UV[cor, 0] / w) * tw
        v = ((F(1) - UV[cor, 1]) / w) * th
        custom0 = (F(1) / w).astype(F)
    else:
        u = UV[cor, 0] * tw
        v = (F(1) - UV[cor, 1]) * th
        custom0 = None
    if S["colors"] is not None:
        col = S["colors"][cor] * mp
    else:
        col = np.broadcast_to(mp, cor.shape + (4,)).astype(F)
    col = col.astype(F).copy()
    if lighting:
        col[..., 0] *= lr[cor]
        col[..., 1] *= lg[cor]
        col[..., 2] *= lb[cor]
    dep = (Z[cor] + margin) / spread
    dep = np.where(dep < F(0), F(0), np.where(dep > F(1), F(1), dep)).astype(F)
    if not S["render_depth"] and S["fog_on"] and S["fog_mode"] in (abi.FOG_ADD, abi.FOG_SUB):
        # FogRange[0] + ((FogRange[1] - FogRange[0]) * 1 - depth), then added to or multiplied
        # into the colour channels (camera.go:1800-1811)
        f0, f1 = S["fog_range"]
        fd = f0 + ((f1 - f0) * F(1) - dep)
        fc = S["fog_color"]
        for k in range(3):
            if S["fog_mode"] == abi.FOG_ADD:
                col[..., k] = col[..., k] + fc[k] * fd
            else:
                col[..., k] = col[..., k] * (fc[k] * fd)
    if not S["render_depth"] and not S["fog_on"]:
        dep = np.zeros_like(dep)  # no depth is computed (the stream holds 0)
    xyuv = np.stack([xs, ys, u, v], -1).astype(F)
    order = order + S["tri_base"]  # mesh-absolute triangle numbers
    if want_custom0:
        return order, xyuv, col.astype(F), dep, custom0
    return order, xyuv, col.astype(F), dep


def scaled_variant():
    """The one-sphere scene (same mesh, colours and rotation) with a non-uniform scale and two more
    point lights: one near enough to light part of the sphere, one that the model-level range skip
    leaves out."""
    from tetra3d_gb300 import abi, scenes
    rng = np.random.Generator(np.random.PCG64(1))
    me = scenes.uv_sphere(32, 16, 1.0)
    me.colors = rng.uniform(0.5, 1.0, (me.nverts, 4)).astype(F)
    lights = [scenes.light(abi.LIGHT_AMBIENT, energy=0.2),
              scenes.light(abi.LIGHT_DIRECTIONAL, energy=1.0,
                           rot=scenes.look_rotation(scenes.unit3(np.array([1, 1, 1], F)))),
              scenes.light(abi.LIGHT_POINT, energy=2.0, rng_=10.0, pos=(2, 2, -3)),
              scenes.light(abi.LIGHT_POINT, color=(0.9, 0.4, 0.2), energy=1.5, rng_=3.0, pos=(-1.5, 0.5, -3.5)),
              scenes.light(abi.LIGHT_POINT, color=(0.2, 0.8, 1.0), energy=3.0, rng_=2.0, pos=(30, 0, -5))]
    sd = scenes.SceneData([me], 1, lights, [[0, 1, 2, 3, 4]], name="uv_sphere_scaled")
    scenes.set_models_trs(sd, 0, [(0, 0, -5)], [(1.3, 0.7, 1.1)], scenes.quat_to_mat(scenes.random_quats(rng, 1)))
    sd.camera = scenes.camera(w=640, h=360, fov=75.0)
    return sd


def volume_variant(lv_mode):
    """The scaled five-light scene plus a light volume around the sphere and the origin (the
    containment test of the per-vertex-with-normal mode reads the zero vector): a 9 x 5 x 17 grid
    of 0.4-unit cells with random colours, offset and light bias, lighting the sphere with the
    material's LightVolumeShadingMode `lv_mode`."""
    from tetra3d_gb300 import abi, scenes
    sd = scaled_variant()
    rng = np.random.Generator(np.random.PCG64(11))
    vmin = np.array([-1.8, -1.0, -6.4], F)
    vmax = np.array([1.8, 1.0, 0.4], F)
    cs = np.array([0.4, 0.4, 0.4], F)
    counts = scenes.light_volume_counts(vmin, vmax, cs)
    cells = np.concatenate([rng.uniform(0.1, 1.0, (int(np.prod(counts)), 3)), np.ones((int(np.prod(counts)), 1))],
                           1).astype(F)
    vol = scenes.light(abi.LIGHT_VOLUME, color=(1.0, 0.9, 0.8), energy=0.7, vol=(vmin, vmax, cs, counts, 0))
    vol.offset[:] = [0.05, -0.1, 0.15]
    vol.bias[:] = [0.02, 0.0, -0.03]
    lights = [sd.lights[i] for i in range(sd.nlights)] + [vol]
    me = sd.meshes[0]
    me.parts[0]["mat"] = dict(me.parts[0]["mat"], lv_shading_mode=lv_mode)
    out = scenes.SceneData([me], 1, lights, [[0, 1, 2, 3, 4, 5]], cells=cells, name=f"uv_sphere_volume{lv_mode}")
    out.mv[:] = sd.mv
    out.camera = sd.camera
    return out


def fog_variant(mode):
    """The scaled five-light scene seen without depth rendering, with the world's fog on in mode
    `mode` (range 0.15-0.85, a blue-grey colour)."""
    sd = scaled_variant()
    cam = sd.camera
    cam.render_depth = 0
    cam.fog_on = 1
    cam.fog_mode = mode
    cam.fog_range[:] = [0.15, 0.85]
    cam.fog_color[:] = [0.4, 0.5, 0.9, 1.0]
    sd.name = f"uv_sphere_fog{mode}"
    return sd


def material_variant(name, light_list=None, lists=None, **mat):
    """The scaled five-light scene with material options `mat` (lighting mode, backface culling,
    sort mode) and, optionally, the model lit by a LightGroup (`light_list` >= 1 of `lists`)."""
    sd = scaled_variant()
    me = sd.meshes[0]
    me.parts[0]["mat"] = dict(me.parts[0]["mat"], **mat)
    if lists is not None:
        sd.lists = lists
    if light_list is not None:
        sd.mv["light_list"][0] = light_list
    sd.name = name
    return sd


def camera_variant(name, tex=None, **cam):
    """The scaled five-light scene with camera options `cam` (perspective-corrected texture
    mapping, vertex snapping, lighting off) and, optionally, a texture size for the material."""
    sd = scaled_variant()
    if tex is not None:
        me = sd.meshes[0]
        me.parts[0]["mat"] = dict(me.parts[0]["mat"], tex_w=float(tex[0]), tex_h=float(tex[1]))
    for k, v in cam.items():
        setattr(sd.camera, k, v)
    sd.name = name
    return sd


def skinned_variant(lighting_mode=0):
    """A tube of 40 rings x 24 segments skinned by a chain of four bones (each vertex blending the
    two nearest, exact 1.0 weights on the bone heights and a few 1.0 weights after a partial one),
    lit by the five-light scene's lights, under material lighting mode `lighting_mode`."""
    from tetra3d_gb300 import abi, scenes
    base = scaled_variant()
    rng = np.random.Generator(np.random.PCG64(9))
    me = scenes.tube_mesh(rings=40, segments=24, height=3.0, radius=0.5)
    me.colors = rng.uniform(0.5, 1.0, (me.nverts, 4)).astype(F)
    me.joints, me.weights = scenes.tube_skin(me, rng, 4)
    me.parts = [dict(tri_start=0, tri_count=me.ntris,
                     mat=scenes.default_material(lighting_mode=lighting_mode, backface_culling=0))]
    lights = [base.lights[i] for i in range(base.nlights)]
    sd = scenes.SceneData([me], 1, lights, [[0, 1, 2, 3, 4]], name=f"skinned_tube{lighting_mode}")
    pos = np.array([(0.3, -1.6, -5.5)], F)
    scenes.set_models_trs(sd, 0, pos, [(1.0, 1.0, 1.0)], scenes.quat_to_mat(scenes.random_quats(rng, 1)))
    sd.mv["skinned"][0] = 1
    sd.mv["bone_first"][0] = 0
    sd.bones = scenes.tube_bones(rng, 1, pos, 4, bend=0.9)
    sd.camera = base.camera
    return sd


def keyed_variant():
    """The scaled five-light sphere with two shape keys: a bulge along the normals (weight 0.6)
    and small random deltas (weight -0.3), with their normal deltas."""
    sd = scaled_variant()
    rng = np.random.Generator(np.random.PCG64(13))
    me = sd.meshes[0]
    bulge = (me.normals * rng.uniform(0.0, 0.25, (me.nverts, 1))).astype(F)
    me.shape_positions = np.stack([bulge, rng.uniform(-0.05, 0.05, bulge.shape).astype(F)])
    me.shape_normals = rng.uniform(-0.1, 0.1, (2, me.nverts, 3)).astype(F)
    me.shape_weights = np.array([0.6, -0.3], F)
    sd.name = "uv_sphere_keyed"
    return sd


def keyed_skinned_variant():
    """The skinned tube with one shape key (weight 0.8) under its skin."""
    sd = skinned_variant()
    rng = np.random.Generator(np.random.PCG64(17))
    me = sd.meshes[0]
    me.shape_positions = (0.08 * rng.standard_normal((1, me.nverts, 3))).astype(F)
    me.shape_normals = (0.05 * rng.standard_normal((1, me.nverts, 3))).astype(F)
    me.shape_weights = np.array([0.8], F)
    sd.name = "skinned_tube_keyed"
    return sd


def plain_colour_variant(shadeless=False):
    """The scaled five-light sphere without a vertex colour channel (the model and material
    colours alone), optionally with the model shadeless."""
    sd = scaled_variant()
    sd.meshes[0].colors = None
    sd.mv["color"][0] = [0.9, 0.7, 0.5, 1.0]
    if shadeless:
        sd.mv["shadeless"][0] = 1
    sd.name = "uv_sphere_plain" + ("_shadeless" if shadeless else "")
    return sd


def nested_variant():
    """The per-vertex light-volume scene with LightVolumeCell.useLights: seven in ten cells each
    light their vertices with one to three of the scene's other lights (ambient, directional and
    point lights, in random order) before their own colour."""
    from tetra3d_gb300 import abi
    sd = volume_variant(abi.LV_PER_VERTEX)
    rng = np.random.Generator(np.random.PCG64(19))
    usable = [0, 1, 2, 3, 4]
    sd.cell_uses = [list(map(int, rng.choice(usable, int(rng.integers(1, 4)), replace=False))) if rng.random() < 0.7
                    else [] for _ in range(sd.ncells)]
    sd.name = "uv_sphere_volume_nested"
    return sd


def cpu_cases():
    """Cases checked against the C++ oracle on the CPU only (the GPU's parity for these camera
    options is checked against the oracle by the feature-scene tests)."""
    return {"c1_pcorrect": camera_variant("c1_pcorrect", tex=(256, 128), perspective_corrected=1),
            "c1_snap": camera_variant("c1_snap", vertex_snapping=64.0),
            "c1_unlit": camera_variant("c1_unlit", lighting_on=0),
            "c1_ortho": camera_variant("c1_ortho", perspective=0, ortho_scale=3.0),
            "c1_ortho_pcorrect": camera_variant("c1_ortho_pcorrect", tex=(64, 64), perspective=0, ortho_scale=2.5,
                                                perspective_corrected=1),
            "skinned_tube": skinned_variant(), "skinned_tube_fixed": skinned_variant(1),
            "c1_shape_keys": keyed_variant(), "skinned_tube_keyed": keyed_skinned_variant(),
            "c1_no_colors": plain_colour_variant(), "c1_no_colors_shadeless": plain_colour_variant(True),
            "c1_volume_nested": nested_variant()}


def is_transparent(md, mat):
    """Model.isTransparent (model.go:1274-1282) with the default source-over blend."""
    from tetra3d_gb300 import abi
    a = F(md["color"][3])
    if mat["present"]:
        mat_t = (mat["transparency_mode"] == abi.TRANSPARENCY_TRANSPARENT or not mat["blend_source_over"] or
                 (mat["transparency_mode"] == abi.TRANSPARENCY_AUTO and F(mat["color"][3]) < F(0.999)))
        return bool(mat_t or (mat["transparency_mode"] != abi.TRANSPARENCY_OPAQUE and a < F(0.999)))
    return bool(a < F(0.999))


def render_frame(sd):
    """Every model of a scene of one-part models, depth rendered: the solid pass draws its render
    pairs in model order, then the transparent pass by RenderOrder ascending and, within one
    order, by the squared camera distance to the model (Vector3.DistanceSquaredTo,
    vector.go:242-247) far to near (camera.go:1343-1457, :2050-2106). Each pair's stream is the
    restatement's for that model and part (nothing for a model outside the frustum). Returns
    [(model, triangle order, xyuv, rgba, depth, part)] in draw order."""
    solids, transparents = [], []
    # Model.DynamicBatchAdd: members draw only inside their owner's pair (opaque batches here)
    batches = {}
    for m in range(sd.nmodels):
        if int(sd.mv[m]["batched"]):
            batches.setdefault(int(sd.mv[m]["batch_owner"]), []).append(m)
    for m in range(sd.nmodels):
        if int(sd.mv[m]["batched"]):
            continue
        md = sd.mv[m]
        nparts = len(sd.meshes[int(md["mesh"])].parts)
        S = scene_inputs(sd, m)
        assert S["render_depth"]
        if m in batches:
            # the owner's pair: its members far to near from the camera (camera.go:2075-2093,
            # Node.DistanceSquaredTo), each culled by its own sphere; the owner draws no mesh
            cp = S["cam_pos"]

            def d2(k):
                wp = np.asarray(sd.mv[k]["transform"], F).reshape(4, 4)[3, :3]
                dx, dy, dz = F(cp[0] - wp[0]), F(cp[1] - wp[1]), F(cp[2] - wp[2])
                return float((dx * dx + dy * dy) + dz * dz)
            dist = [d2(k) for k in batches[m]]
            assert len(set(dist)) == len(dist), "sort.Slice is not stable: keep the distances distinct"
            for k in sorted(batches[m], key=d2, reverse=True):
                for q in range(len(sd.meshes[int(sd.mv[k]["mesh"])].parts)):
                    solids.append((k,) + tuple(render(scene_inputs(sd, k, q))) + (q,))
            continue
        for q in range(nparts):  # one render pair per mesh part, in part order
            mat = sd.meshes[int(md["mesh"])].parts[q]["mat"]
            item = (m,) + tuple(render(scene_inputs(sd, m, q))) + (q,)
            if is_transparent(md, mat):
                wp = np.asarray(md["transform"], F).reshape(4, 4)[3, :3]  # Model.WorldPosition
                cp = S["cam_pos"]
                dx, dy, dz = F(cp[0] - wp[0]), F(cp[1] - wp[1]), F(cp[2] - wp[2])
                dist = (dx * dx + dy * dy) + dz * dz
                order = int(mat["render_order"]) if mat["present"] else 0
                transparents.append(((order, -float(dist)), item))
            else:
                solids.append(item)
    transparents.sort(key=lambda t: t[0])  # a strict weak order: any stable sort agrees
    return solids + [t[1] for t in transparents]


def multi_model_variant():
    """Six spheres of the five-light scene's mesh: different positions (one behind the camera and
    one far to the side, both culled by SphereInFrustum), non-uniform scales, rotations and model
    colours, half of them lit by a LightGroup of three lights."""
    from tetra3d_gb300 import scenes
    base = scaled_variant()
    rng = np.random.Generator(np.random.PCG64(5))
    lights = [base.lights[i] for i in range(base.nlights)]
    sd = scenes.SceneData([base.meshes[0]], 6, lights, [[0, 1, 2, 3, 4], [0, 2, 3]], name="six_spheres")
    pos = np.array([(0, 0, -5), (-2.2, 0.8, -7), (2.5, -0.6, -9), (0, 0, 6), (40, 0, -6), (1.0, 1.4, -4)], F)
    scl = rng.uniform(0.5, 1.4, (6, 3)).astype(F)
    rot = scenes.quat_to_mat(scenes.random_quats(rng, 6))
    scenes.set_models_trs(sd, np.zeros(6, np.uint32), pos, scl, rot)
    sd.mv["color"] = np.concatenate([rng.uniform(0.6, 1.0, (6, 3)), np.ones((6, 1))], 1).astype(F)
    sd.mv["light_list"] = np.array([-1, 1, -1, 1, -1, 1], np.int32)
    sd.camera = base.camera
    return sd


def cases():
    from tetra3d_gb300 import abi, scenes
    return {"c1": scenes.uv_sphere_scene(1), "c1_scaled_5lights": scaled_variant(),
            "c1_volume_vertex": volume_variant(abi.LV_PER_VERTEX),
            "c1_volume_normal": volume_variant(abi.LV_PER_VERTEX_WITH_NORMAL),
            "c1_volume_object": volume_variant(abi.LV_PER_OBJECT),
            "c1_fog_add": fog_variant(abi.FOG_ADD), "c1_fog_sub": fog_variant(abi.FOG_SUB),
            "c1_fixed_normals": material_variant("c1_fixed_normals", lighting_mode=abi.LIGHTING_FIXED_NORMALS),
            "c1_double_sided_nocull": material_variant("c1_double_sided_nocull", lighting_mode=abi.LIGHTING_DOUBLE_SIDED,
                                                       backface_culling=0, sort_mode=abi.SORT_FRONT_TO_BACK),
            "c1_unsorted_group": material_variant("c1_unsorted_group", light_list=1,
                                                  lists=[[0, 1, 2, 3, 4], [0, 2, 3]], sort_mode=abi.SORT_NONE)}


def input_digest(S):
    h = hashlib.sha256()
    for k in ("positions", "normals", "uvs", "colors", "indices", "model_pos", "model_scale", "model_rot",
              "model_color", "mat_color", "cam_rot"):
        if S[k] is not None:
            h.update(np.ascontiguousarray(S[k]).tobytes())
    for L in S["lights"]:
        h.update(np.asarray([L["type"]], np.int64).tobytes())
        h.update(np.asarray([*L["color"], L["energy"], L["range"], *L["world_pos"]], F).tobytes())
        h.update(L["world_rot"].tobytes())
        if L["type"] == 3:  # a light volume: its grid and cells
            h.update(np.concatenate([L["vol_min"], L["vol_max"], L["cell_size"], L["offset"], L["bias"]]).tobytes())
            h.update(np.asarray([*L["cell_count"], L["cell_first"], S["lv_mode"]], np.int64).tobytes())
            h.update(np.ascontiguousarray(S["cells"]).tobytes())
    h.update(np.asarray([*S["cam_pos"], S["fov"], S["near"], S["far"], S["depth_margin"]], F).tobytes())
    h.update(np.asarray([S["width"], S["height"], S["sort_mode"], S["backface"]], np.int64).tobytes())
    if S["lighting_mode"]:
        h.update(np.asarray([S["lighting_mode"]], np.int64).tobytes())
    if S["pcorrect"] or S["snap"] > F(0) or not S["lighting_on"]:
        h.update(np.asarray([S["pcorrect"], S["lighting_on"]], np.int64).tobytes())
        h.update(np.asarray([S["snap"], *S["tex"]], F).tobytes())
    if not S["perspective"]:
        h.update(np.asarray([0, S["ortho_scale"]], F).tobytes())
    if S["skinned"]:
        h.update(np.asarray([S["bone_first"]], np.int64).tobytes())
        for k in ("joints", "weights", "bones"):
            h.update(np.ascontiguousarray(S[k]).tobytes())
    if S["shape_weights"] is not None:
        for k in ("shape_positions", "shape_normals", "shape_weights"):
            h.update(np.ascontiguousarray(S[k]).tobytes())
    if S["cell_uses"] is not None:
        h.update(repr(S["cell_uses"]).encode())
    if S["colors"] is None or S["shadeless"]:
        h.update(np.asarray([S["colors"] is None, S["shadeless"]], np.int64).tobytes())
    if S["fog_on"] or not S["render_depth"]:  # the fog and depth options (unchanged digests otherwise)
        h.update(np.asarray([S["render_depth"], S["fog_on"], S["fog_mode"]], np.int64).tobytes())
        h.update(np.concatenate([S["fog_range"], S["fog_color"]]).tobytes())
    return h.hexdigest()


def transparent_variant():
    """The six-sphere frame with two models half transparent (model alpha 0.5): they move to the
    transparent pass, far one first."""
    sd = multi_model_variant()
    sd.mv["color"][1, 3] = 0.5
    sd.mv["color"][5, 3] = 0.5
    sd.name = "six_spheres_transparent"
    return sd


def batch_variant():
    """Six spheres, four of them members of model 0's dynamic batch (one behind the camera, culled
    inside the batch; two lit by a LightGroup), and one model drawn on its own after the batch."""
    from tetra3d_gb300 import scenes
    base = scaled_variant()
    rng = np.random.Generator(np.random.PCG64(23))
    lights = [base.lights[i] for i in range(base.nlights)]
    sd = scenes.SceneData([base.meshes[0]], 6, lights, [[0, 1, 2, 3, 4], [0, 2, 3]], name="batch6")
    pos = np.array([(0, 0, -5), (-2.0, 0.5, -8), (1.5, -0.5, -4.5), (2.5, 0.8, -11), (0, 0, 7), (-1.2, -1.0, -6)], F)
    scl = rng.uniform(0.4, 1.0, (6, 3)).astype(F)
    rot = scenes.quat_to_mat(scenes.random_quats(rng, 6))
    scenes.set_models_trs(sd, np.zeros(6, np.uint32), pos, scl, rot)
    sd.mv["batched"][1:5] = 1
    sd.mv["batch_owner"][1:5] = 0
    sd.mv["batch_part"][1:5] = 0
    sd.mv["light_list"][[2, 3]] = 1
    sd.camera = base.camera
    return sd


def two_part_variant():
    """Three models of a sphere cut into two mesh parts: the top half opaque with the default
    material, the bottom half with fixed-normal lighting, front-to-back sorting and a material
    alpha of 0.6 (so it is drawn in the transparent pass, far to near)."""
    import copy
    from tetra3d_gb300 import abi, scenes
    base = scaled_variant()
    rng = np.random.Generator(np.random.PCG64(29))
    me = copy.deepcopy(base.meshes[0])
    half = me.ntris // 2
    m0 = dict(me.parts[0]["mat"])
    m1 = dict(m0, lighting_mode=abi.LIGHTING_FIXED_NORMALS, sort_mode=abi.SORT_FRONT_TO_BACK, color=(1, 1, 1, 0.6))
    me.parts = [dict(tri_start=0, tri_count=half, mat=m0), dict(tri_start=half, tri_count=me.ntris - half, mat=m1)]
    lights = [base.lights[i] for i in range(base.nlights)]
    sd = scenes.SceneData([me], 3, lights, [[0, 1, 2, 3, 4], [0, 2, 3]], name="two_parts")
    pos = np.array([(0, 0, -6), (-1.8, 0.6, -4.5), (1.6, -0.4, -8)], F)
    scl = rng.uniform(0.6, 1.2, (3, 3)).astype(F)
    scenes.set_models_trs(sd, np.zeros(3, np.uint32), pos, scl, scenes.quat_to_mat(scenes.random_quats(rng, 3)))
    sd.mv["light_list"][1] = 1
    sd.camera = base.camera
    return sd


def frame_cases():
    """Multi-model cases, checked against the C++ oracle pair by pair."""
    return {"six_spheres": multi_model_variant(), "six_spheres_transparent": transparent_variant(),
            "batch6": batch_variant(), "two_parts": two_part_variant()}


def main():
    out = {}
    for name, sd in frame_cases().items():
        parts = render_frame(sd)
        out[f"{name}_models"] = np.array([p[0] for p in parts], np.uint32)
        out[f"{name}_parts"] = np.array([p[5] for p in parts], np.uint32)
        out[f"{name}_counts"] = np.array([len(p[1]) for p in parts], np.uint32)
        out[f"{name}_order"] = np.concatenate([p[1] for p in parts]).astype(np.uint32)
        for k, i in (("xyuv", 2), ("rgba", 3), ("depth", 4)):
            out[f"{name}_{k}"] = np.concatenate([p[i] for p in parts])
        out[f"{name}_digest"] = np.frombuffer(bytes.fromhex(
            hashlib.sha256("".join(input_digest(scene_inputs(sd, m)) for m in range(sd.nmodels)).encode()).hexdigest()),
            np.uint8)
        print(name, "visible per model", out[f"{name}_counts"].tolist())
    for name, sd in {**cases(), **cpu_cases()}.items():
        S = scene_inputs(sd)
        order, xyuv, rgba, depth, custom0 = render(S, want_custom0=True)
        out[f"{name}_order"] = order.astype(np.uint32)
        out[f"{name}_xyuv"] = xyuv
        out[f"{name}_rgba"] = rgba
        out[f"{name}_depth"] = depth
        if custom0 is not None:
            out[f"{name}_custom0"] = custom0
        out[f"{name}_digest"] = np.frombuffer(bytes.fromhex(input_digest(S)), np.uint8)
        print(name, "visible", len(order))
    np.savez_compressed(os.path.join(HERE, "c1_whole_path.npz"), **out)


if __name__ == "__main__":
    main()
