"""Seeded synthetic scenes for the vertex stage and their C descriptors.

Every array is float32 and every derived matrix is computed with Tetra3D's
binary32 operation order (no fused multiply-add), so the same SceneData fed to
the CUDA library and to the oracle describes bit-identical inputs.

Workloads (sizes as named in the benchmark configuration):
  uv_sphere_scene   one UV sphere, 32 segments x 16 rings (544 V / 960 T)
  cubes_scene       1000 unit cubes (24 V / 12 T each), 8 point lights
  terrain_scene     1024x1024-vertex value-noise grid split into 4 quadrant
                    models with 4 light groups, 16 point + 1 directional + 2 box lights
  batched_scene     4096 models, vertex counts log-uniform in [24, 65536]
  serving scenes    64 resident scenes drawn from the three above
"""
import ctypes as C
import math

import numpy as np

from . import abi

F32 = np.float32
PI32 = F32(math.pi)  # math32.Pi = float32(math.Pi)


# --------------------------------------------------------------- matrices ----
def ident(n=None):
    if n is None:
        return np.eye(4, dtype=F32)
    return np.broadcast_to(np.eye(4, dtype=F32), (n, 4, 4)).copy()


def mult(a, b):
    """Matrix4.Mult with the reference's left-to-right sums (matrix_none.go:6-32), batched."""
    a = np.asarray(a, F32)
    b = np.asarray(b, F32)
    out = np.empty(np.broadcast_shapes(a.shape, b.shape), F32)
    for i in range(4):
        for j in range(4):
            s = a[..., i, 0] * b[..., 0, j]
            s = s + a[..., i, 1] * b[..., 1, j]
            s = s + a[..., i, 2] * b[..., 2, j]
            s = s + a[..., i, 3] * b[..., 3, j]
            out[..., i, j] = s
    return out


def translate(x, y, z):
    m = ident()
    m[3, 0], m[3, 1], m[3, 2] = F32(x), F32(y), F32(z)
    return m


def scale_m(x, y, z):
    m = ident()
    m[0, 0], m[1, 1], m[2, 2] = F32(x), F32(y), F32(z)
    return m


def unit3(v):
    """Vector3.Unit (vector.go:258-266) on float32 (..., 3)."""
    v = np.asarray(v, F32)
    ln = (v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1] + v[..., 2] * v[..., 2]).astype(F32)
    ln = np.sqrt(ln.astype(np.float64)).astype(F32)
    keep = (ln < F32(1e-8)) | (ln == F32(1))
    safe = np.where(keep, F32(1), ln)
    out = (v / safe[..., None]).astype(F32)
    return np.where(keep[..., None], v, out).astype(F32)


def rotate(x, y, z, angle):
    """NewMatrix4Rotate (matrix.go:101-128); Sin/Cos in float64 like math32."""
    if x == 0 and y == 0 and z == 0:
        y = 1
    v = unit3(np.array([x, y, z], F32))
    s = F32(math.sin(float(F32(angle))))
    c = F32(math.cos(float(F32(angle))))
    m = F32(1) - c
    X, Y, Z = v
    r = ident()
    r[0, 0] = m * X * X + c
    r[0, 1] = m * X * Y + Z * s
    r[0, 2] = m * Z * X - Y * s
    r[1, 0] = m * X * Y - Z * s
    r[1, 1] = m * Y * Y + c
    r[1, 2] = m * Y * Z + X * s
    r[2, 0] = m * Z * X + Y * s
    r[2, 1] = m * Y * Z - X * s
    r[2, 2] = m * Z * Z + c
    return r


def quat_to_mat(q):
    """Quaternion.ToMatrix4 (quaternion.go:135-182), batched over (n, 4) = (x, y, z, w)."""
    q = np.asarray(q, F32).reshape(-1, 4)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    n = q.shape[0]
    m1 = ident(n)
    m2 = ident(n)
    m1[:, 0] = np.stack([w, z, -y, x], 1)
    m1[:, 1] = np.stack([-z, w, x, y], 1)
    m1[:, 2] = np.stack([y, -x, w, z], 1)
    m1[:, 3] = np.stack([-x, -y, -z, w], 1)
    m2[:, 0] = np.stack([w, z, -y, -x], 1)
    m2[:, 1] = np.stack([-z, w, x, -y], 1)
    m2[:, 2] = np.stack([y, -x, w, -z], 1)
    m2[:, 3] = np.stack([x, y, z, w], 1)
    return mult(m1, m2)


def random_quats(rng, n):
    """Uniformly distributed unit quaternions (Shoemake's subgroup method)."""
    u = rng.random((n, 3))
    a = np.sqrt(1 - u[:, 0])
    b = np.sqrt(u[:, 0])
    q = np.stack([a * np.sin(2 * np.pi * u[:, 1]), a * np.cos(2 * np.pi * u[:, 1]),
                  b * np.sin(2 * np.pi * u[:, 2]), b * np.cos(2 * np.pi * u[:, 2])], 1)
    return q.astype(F32)


def trs(pos, scl, rot):
    """Node.Transform of a parentless node: Scale * Rotation * Translate (node.go:583-585), batched."""
    pos = np.asarray(pos, F32).reshape(-1, 3)
    scl = np.asarray(scl, F32).reshape(-1, 3)
    rot = np.asarray(rot, F32).reshape(-1, 4, 4)
    n = max(pos.shape[0], scl.shape[0], rot.shape[0])
    S = ident(n)
    S[:, 0, 0], S[:, 1, 1], S[:, 2, 2] = scl[:, 0], scl[:, 1], scl[:, 2]
    T = ident(n)
    T[:, 3, 0], T[:, 3, 1], T[:, 3, 2] = pos[:, 0], pos[:, 1], pos[:, 2]
    return mult(mult(S, rot), T)


def look_rotation(forward_row):
    """A rotation whose row 2 (Forward) is the given unit vector; rows 0/1 complete a right-handed basis."""
    z = unit3(np.asarray(forward_row, F32))
    up = np.array([0, 1, 0], F32) if abs(float(z[1])) < 0.99 else np.array([1, 0, 0], F32)
    x = unit3(np.cross(up, z).astype(F32))
    y = np.cross(z, x).astype(F32)
    r = ident()
    r[0, :3], r[1, :3], r[2, :3] = x, y, z
    return r


# ------------------------------------------------------------------ meshes ----
def default_material(**kw):
    m = dict(color=(1, 1, 1, 1), tex_w=0.0, tex_h=0.0, present=1, backface_culling=1,
             sort_mode=abi.SORT_BACK_TO_FRONT, lighting_mode=abi.LIGHTING_DEFAULT, lv_shading_mode=abi.LV_PER_VERTEX,
             shadeless=0, visible=1, transparency_mode=abi.TRANSPARENCY_AUTO, blend_source_over=1, render_order=0,
             texture=0, texture_filter=0, texture_map_mode=0, texture_map_scale=(1.0, 1.0))
    m.update(kw)
    return m


class MeshData:
    """A mesh's SoA streams. Optional: shape keys (shape_positions / shape_normals (K, V, 3) deltas,
    shape_weights (K,)) and skinning joints / weights (V, 4)."""

    def __init__(self, positions, normals, uvs, indices, colors=None, parts=None, dims=None):
        self.positions = np.ascontiguousarray(positions, F32).reshape(-1, 3)
        self.normals = np.ascontiguousarray(normals, F32).reshape(-1, 3)
        self.uvs = np.ascontiguousarray(uvs, F32).reshape(-1, 2)
        self.colors = None if colors is None else np.ascontiguousarray(colors, F32).reshape(-1, 4)
        self.indices = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        T = self.indices.shape[0]
        self.parts = parts if parts is not None else [dict(tri_start=0, tri_count=T, mat=default_material())]
        self.dims = dims  # None: UpdateDimensions
        self.shape_positions = self.shape_normals = self.shape_weights = None
        self.joints = self.weights = None
        self.auto_subdivide = 0  # Mesh.SetAutoSubdivide

    @property
    def nverts(self):
        return self.positions.shape[0]

    @property
    def ntris(self):
        return self.indices.shape[0]


def flat_normals_like_autonormal(positions, indices):
    """Mesh.AutoNormal (mesh.go:755-764): every vertex of a triangle gets the triangle normal, in triangle order."""
    p = positions.astype(F32)
    n = np.zeros_like(p)
    a, b, c = p[indices[:, 0]], p[indices[:, 1]], p[indices[:, 2]]
    v0 = (b - a).astype(F32)
    v1 = (c - b).astype(F32)
    cr = np.stack([v0[:, 1] * v1[:, 2] - v1[:, 1] * v0[:, 2],
                   v0[:, 2] * v1[:, 0] - v1[:, 2] * v0[:, 0],
                   v0[:, 0] * v1[:, 1] - v1[:, 0] * v0[:, 1]], 1).astype(F32)
    tn = unit3(cr)
    for k in range(3):  # later triangles overwrite earlier ones, as in the reference loop
        n[indices[:, k]] = tn
    # vectorised assignment keeps the last writer per vertex only within one column; redo exactly in order
    for t in range(indices.shape[0]):
        for k in range(3):
            n[indices[t, k]] = tn[t]
    return n


def cube_mesh(w=1.0, h=1.0, d=1.0):
    """NewCubeMesh (mesh.go:1251-1342): 24 vertices, 12 triangles, flat normals."""
    w, h, d = F32(w) / F32(2), F32(h) / F32(2), F32(d) / F32(2)
    v = [(-w, h, -d, 0, 0), (w, h, d, 1, 1), (w, h, -d, 1, 0), (-w, h, d, 0, 1),
         (w, -h, -d, 1, 0), (w, -h, d, 1, 1), (-w, -h, -d, 0, 0), (-w, -h, d, 0, 1),
         (-w, h, d, 0, 0), (w, -h, d, 1, 1), (w, h, d, 1, 0), (-w, -h, d, 0, 1),
         (w, h, -d, 1, 0), (w, -h, -d, 1, 1), (-w, h, -d, 0, 0), (-w, -h, -d, 0, 1),
         (w, h, -d, 1, 0), (w, h, d, 1, 1), (w, -h, -d, 0, 0), (w, -h, d, 0, 1),
         (-w, -h, -d, 0, 0), (-w, h, d, 1, 1), (-w, h, -d, 1, 0), (-w, -h, d, 0, 1)]
    arr = np.array(v, F32)
    idx = np.array([0, 1, 2, 3, 1, 0, 4, 5, 6, 6, 5, 7, 8, 9, 10, 11, 9, 8,
                    12, 13, 14, 14, 13, 15, 16, 17, 18, 18, 17, 19, 20, 21, 22, 23, 21, 20], np.uint32).reshape(-1, 3)
    pos = arr[:, :3]
    nrm = flat_normals_like_autonormal(pos, idx)
    return MeshData(pos, nrm, arr[:, 3:5], idx)


def _orient_outward(pos, idx, center=None):
    """Flips triangles whose geometric normal points towards `center` so outward faces wind CCW."""
    c = np.zeros(3, F32) if center is None else np.asarray(center, F32)
    a, b, cc = pos[idx[:, 0]], pos[idx[:, 1]], pos[idx[:, 2]]
    nrm = np.cross(b - a, cc - b)
    out = ((a + b + cc) / 3 - c)
    flip = (nrm * out).sum(1) < 0
    idx = idx.copy()
    idx[flip, 1], idx[flip, 2] = idx[flip, 2].copy(), idx[flip, 1].copy()
    return idx


def uv_sphere(segments=32, rings=16, radius=1.0):
    """A UV sphere built with the NewMesh/AddVertices/AddTriangles recipe (mesh.go:1230-1248):
    (rings+1) x segments vertices, smooth normals, poles as single triangles."""
    r = np.arange(rings + 1)[:, None]
    s = np.arange(segments)[None, :]
    th = np.pi * r / rings + 0 * s
    ph = 2 * np.pi * s / segments + 0 * r
    pos = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1).reshape(-1, 3)
    pos = (pos * radius).astype(F32)
    nrm = unit3(pos)
    uv = np.stack([(s / segments + 0 * r), (r / rings + 0 * s)], -1).reshape(-1, 2).astype(F32)
    tris = []
    for i in range(rings):
        for j in range(segments):
            a = i * segments + j
            b = i * segments + (j + 1) % segments
            c = (i + 1) * segments + j
            d = (i + 1) * segments + (j + 1) % segments
            if i != 0:
                tris.append((a, b, c))
            if i != rings - 1:
                tris.append((b, d, c))
    idx = _orient_outward(pos, np.array(tris, np.uint32))
    return MeshData(pos, nrm, uv, idx)


def icosphere(level):
    """Icosahedron subdivided `level` times, vertices pushed to the unit sphere, flat normals (AutoNormal)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(v, np.float64) for v in verts]
    for _ in range(level):
        cache = {}

        def mid(i, j):
            key = (min(i, j), max(i, j))
            if key not in cache:
                verts.append((verts[i] + verts[j]) / 2)
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    pos = np.array(verts)
    pos = (pos / np.linalg.norm(pos, axis=1, keepdims=True)).astype(F32)
    idx = _orient_outward(pos, np.array(faces, np.uint32))
    nrm = flat_normals_like_autonormal(pos, idx) if len(faces) < 4096 else unit3(pos)
    uv = np.zeros((pos.shape[0], 2), F32)
    uv[1::3, 0] = 1
    uv[2::3, 1] = 1
    return MeshData(pos, nrm, uv, idx)


def value_noise(rng_seed, x, z, octaves=4):
    """Seeded 2D value noise: random lattice values, smoothstep-bilinear, `octaves` octaves (float64)."""
    total = np.zeros_like(x, dtype=np.float64)
    amp, freq, norm = 1.0, 1.0, 0.0
    for o in range(octaves):
        rng = np.random.Generator(np.random.PCG64([rng_seed, o]))
        xs, zs = x * freq, z * freq
        x0, z0 = np.floor(xs).astype(np.int64), np.floor(zs).astype(np.int64)
        gx0, gz0 = x0.min(), z0.min()
        lat = rng.random((int(x0.max() - gx0) + 2, int(z0.max() - gz0) + 2)) * 2 - 1
        fx, fz = xs - x0, zs - z0
        sx, sz = fx * fx * (3 - 2 * fx), fz * fz * (3 - 2 * fz)
        i, j = x0 - gx0, z0 - gz0
        v00, v10, v01, v11 = lat[i, j], lat[i + 1, j], lat[i, j + 1], lat[i + 1, j + 1]
        total += amp * ((v00 * (1 - sx) + v10 * sx) * (1 - sz) + (v01 * (1 - sx) + v11 * sx) * sz)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def grid_mesh(nx, nz, extent_x, extent_z, heights, x0=0.0, z0=0.0):
    """A grid of nx x nz vertices (row-major in z), NewPlaneMesh's triangle order (mesh.go:1533-1589)."""
    xs = (x0 + np.arange(nx) * (extent_x / max(nx - 1, 1))).astype(np.float64)
    zs = (z0 + np.arange(nz) * (extent_z / max(nz - 1, 1))).astype(np.float64)
    X, Z = np.meshgrid(xs, zs)
    H = heights(X, Z)
    pos = np.stack([X, H, Z], -1).reshape(-1, 3).astype(F32)
    # central finite differences
    dx, dz = extent_x / max(nx - 1, 1), extent_z / max(nz - 1, 1)
    hp = np.pad(H, 1, mode="edge")
    gx = (hp[1:-1, 2:] - hp[1:-1, :-2]) / (2 * dx)
    gz = (hp[2:, 1:-1] - hp[:-2, 1:-1]) / (2 * dz)
    nrm = np.stack([-gx, np.ones_like(gx), -gz], -1)
    nrm = (nrm / np.linalg.norm(nrm, axis=-1, keepdims=True)).reshape(-1, 3).astype(F32)
    uv = np.stack([(X - X.min()) / max(extent_x, 1e-9), (Z - Z.min()) / max(extent_z, 1e-9)], -1).reshape(-1, 2).astype(F32)
    q = (np.arange(nz - 1)[:, None] * nx + np.arange(nx - 1)[None, :]).reshape(-1)
    idx = np.stack([q + 1, q + nx, q + nx + 1, q, q + nx, q + 1], 1).reshape(-1, 3).astype(np.uint32)
    return MeshData(pos, nrm, uv, idx)


# ------------------------------------------------------------------ scenes ----
class SceneData:
    """Meshes, models, lights and light lists of one scene plus a default camera.

    light list 0 is the scene light list in Render order; lists 1.. are LightGroups.
    """

    def __init__(self, meshes, nmodels, lights, lists, cells=None, name=""):
        self.name = name
        self.meshes = meshes
        self.models = (abi.ModelDesc * max(1, nmodels))()
        self.nmodels = nmodels
        self.mv = np.ctypeslib.as_array(self.models)[:nmodels]
        self.lights = (abi.LightDesc * max(1, len(lights)))(*lights)
        self.nlights = len(lights)
        self.lists = [list(map(int, l)) for l in lists]
        self.cells = np.zeros((1, 4), F32) if cells is None or len(cells) == 0 else np.ascontiguousarray(cells, F32)
        self.ncells = 0 if cells is None else len(cells)
        self.camera = None
        self.bones = None  # (NB, 16) Node.boneInfluence matrices
        self.subdivision_levels = None  # (L, 2) AutoSubdivisionLevel: DistanceSquared, MaximumTriangleSize
        self.cell_uses = None           # per light-volume cell: light indices (LightVolumeCell.useLights)
        self.max_subdivisions = 0       # Library.maxAutoSubdivisionCount (0: 3)
        self.meta = {}
        self._keep = []

    def desc(self):
        keep = []
        md = (abi.MeshDesc * max(1, len(self.meshes)))()
        for i, m in enumerate(self.meshes):
            pa = (abi.PartDesc * max(1, len(m.parts)))()
            for k, p in enumerate(m.parts):
                pa[k].tri_start = p["tri_start"]
                pa[k].tri_count = p["tri_count"]
                mat = p["mat"]
                for f, v in mat.items():
                    if f == "color":
                        pa[k].mat.color[:] = [float(c) for c in v]
                    elif f == "billboard_lock":
                        pa[k].mat.billboard_lock[:] = [int(c) for c in v]
                    elif f == "texture_map_scale":
                        pa[k].mat.texture_map_scale[:] = [float(c) for c in v]
                    else:
                        setattr(pa[k].mat, f, v)
            keep.append(pa)
            d = md[i]
            d.positions, d.normals, d.uvs = abi.fptr(m.positions), abi.fptr(m.normals), abi.fptr(m.uvs)
            d.colors = abi.fptr(m.colors) if m.colors is not None else None
            d.indices = abi.uptr(m.indices)
            d.parts = C.cast(pa, C.POINTER(abi.PartDesc))
            d.num_vertices, d.num_triangles, d.num_parts = m.nverts, m.ntris, len(m.parts)
            if m.dims is not None:
                d.has_dimensions = 1
                d.dim_min[:] = [float(x) for x in m.dims[0]]
                d.dim_max[:] = [float(x) for x in m.dims[1]]
            if m.shape_weights is not None and len(m.shape_weights):
                sp = np.ascontiguousarray(m.shape_positions, F32)
                sn = np.ascontiguousarray(m.shape_normals, F32)
                sw = np.ascontiguousarray(m.shape_weights, F32)
                keep += [sp, sn, sw]
                d.shape_positions, d.shape_normals, d.shape_weights = abi.fptr(sp), abi.fptr(sn), abi.fptr(sw)
                d.num_shape_keys = len(sw)
            d.auto_subdivide = int(m.auto_subdivide)
            if m.joints is not None:
                jt = np.ascontiguousarray(m.joints, np.uint32)
                wt = np.ascontiguousarray(m.weights, F32)
                keep += [jt, wt]
                d.joints, d.weights = abi.uptr(jt), abi.fptr(wt)
        offs = np.zeros(len(self.lists) + 1, np.uint32)
        for i, l in enumerate(self.lists):
            offs[i + 1] = offs[i] + len(l)
        items = np.array([x for l in self.lists for x in l] or [0], np.uint32)
        keep += [md, offs, items]
        sd = abi.SceneDesc()
        sd.meshes = C.cast(md, C.POINTER(abi.MeshDesc))
        sd.models = C.cast(self.models, C.POINTER(abi.ModelDesc))
        sd.lights = C.cast(self.lights, C.POINTER(abi.LightDesc))
        sd.volume_cells = abi.fptr(self.cells)
        sd.list_offsets = abi.uptr(offs)
        sd.list_items = abi.uptr(items)
        sd.num_meshes, sd.num_models, sd.num_lights = len(self.meshes), self.nmodels, self.nlights
        sd.num_volume_cells, sd.num_lists = self.ncells, len(self.lists)
        if self.bones is not None and len(self.bones):
            bones = np.ascontiguousarray(self.bones, F32).reshape(-1, 16)
            keep.append(bones)
            sd.bones, sd.num_bones = abi.fptr(bones), bones.shape[0]
        if self.subdivision_levels is not None and len(self.subdivision_levels):
            lev = np.ascontiguousarray(self.subdivision_levels, F32).reshape(-1, 2)
            keep.append(lev)
            sd.subdivision_levels, sd.num_subdivision_levels = abi.fptr(lev), lev.shape[0]
        sd.max_subdivisions = int(self.max_subdivisions)
        if self.cell_uses is not None:
            offs = np.zeros(self.ncells + 1, np.uint32)
            for c in range(self.ncells):
                offs[c + 1] = offs[c] + len(self.cell_uses[c])
            items = np.array([x for c in range(self.ncells) for x in self.cell_uses[c]] or [0], np.uint32)
            keep += [offs, items]
            sd.cell_use_offsets, sd.cell_use_items = abi.uptr(offs), abi.uptr(items)
        self._keep = keep
        return sd

    def total_tris(self):
        return sum(self.meshes[int(m)].ntris for m in self.mv["mesh"])

    def total_verts(self):
        return sum(self.meshes[int(m)].nverts for m in self.mv["mesh"])


def set_models_trs(sd, mesh, pos, scl, rot, color=(1, 1, 1, 1), light_list=-1, frustum=1, step=None):
    n = sd.nmodels
    mv = sd.mv
    mv["mesh"] = np.asarray(mesh, np.uint32).reshape(-1) if np.ndim(mesh) else mesh
    mv["visible"] = 1
    mv["frustum_culling"] = frustum
    mv["shadeless"] = 0
    mv["light_list"] = light_list
    mv["use_trs"] = 1
    mv["color"] = np.broadcast_to(np.asarray(color, F32), (n, 4))
    rot = np.asarray(rot, F32).reshape(n, 4, 4)
    pos = np.asarray(pos, F32).reshape(n, 3)
    scl = np.asarray(scl, F32).reshape(n, 3)
    mv["position"] = pos
    mv["scale"] = scl
    mv["rotation"] = rot.reshape(n, 16)
    M = trs(pos, scl, rot)
    mv["transform"] = M.reshape(n, 16)
    mv["world_rotation"] = rot.reshape(n, 16)
    mv["rotate_step"] = (ident(n) if step is None else np.asarray(step, F32).reshape(n, 4, 4)).reshape(n, 16)


def light(kind, color=(1, 1, 1), energy=1.0, rng_=0.0, pos=(0, 0, 0), rot=None, vol=None):
    L = abi.LightDesc()
    L.type = kind
    L.color[:] = [float(color[0]), float(color[1]), float(color[2]), 1.0]
    L.energy = float(energy)
    L.range = float(rng_)
    r = ident() if rot is None else np.asarray(rot, F32)
    M = mult(r, translate(*pos))
    L.transform[:] = M.reshape(16).tolist()
    L.world_rotation[:] = r.reshape(16).tolist()
    if vol is not None:
        vmin, vmax, cell, counts, first = vol
        L.vol_min[:] = [float(x) for x in vmin]
        L.vol_max[:] = [float(x) for x in vmax]
        L.cell_size[:] = [float(x) for x in cell]
        L.cell_count[:] = [int(x) for x in counts]
        L.cell_first = first
    return L


def light_volume_counts(vmin, vmax, cell):
    """LightVolumeResize's cell counts (light.go:485-513): float32 accumulation loops."""
    counts = []
    for a in range(3):
        lo, hi, cs = F32(vmin[a]), F32(vmax[a]), F32(cell[a])
        k = 0
        x = lo + F32(cs / F32(2))
        while x <= hi - F32(cs / F32(2)):
            k += 1
            x = F32(x + cs)
        counts.append(k)
    return counts


def camera(pos=(0, 0, 0), rot=None, w=640, h=360, fov=60.0, near=0.1, far=100.0, perspective=1,
           render_depth=1, lighting_on=1, fog_on=1, fog_mode=abi.FOG_ADD, ortho_scale=20.0):
    c = abi.CameraDesc()
    r = ident() if rot is None else np.asarray(rot, F32)
    M = trs(np.asarray(pos, F32), np.ones(3, F32), r)[0]
    c.transform[:] = M.reshape(16).tolist()
    c.world_rotation[:] = r.reshape(16).tolist()
    c.width, c.height = int(w), int(h)
    c.perspective, c.render_depth, c.perspective_corrected = perspective, render_depth, 0
    c.lighting_on, c.fog_on, c.fog_mode = lighting_on, fog_on, fog_mode
    c.fov_y, c.near_plane, c.far_plane = float(fov), float(near), float(far)
    c.ortho_scale, c.depth_margin = float(ortho_scale), 0.04
    c.fog_range[:] = [0.0, 1.0]
    c.fog_color[:] = [0.0, 0.0, 0.0, 0.0]
    return c


def deg2rad(deg):
    """math32.ToRadians (math32.go:14-16)."""
    return F32(math.pi) * F32(deg) / F32(180)


# ------------------------------------------------------------- workloads ----
def uv_sphere_scene(seed=1, w=640, h=360):
    """One UV sphere (radius 1, 32 x 16), RGBA vertex colours in [0.5, 1], random rotation at (0,0,-5);
    640x360 FOV 75, ambient 0.2, a directional light along -(1,1,1), a point light at (2,2,-3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    me = uv_sphere(32, 16, 1.0)
    me.colors = rng.uniform(0.5, 1.0, (me.nverts, 4)).astype(F32)
    lights = [light(abi.LIGHT_AMBIENT, energy=0.2),
              light(abi.LIGHT_DIRECTIONAL, energy=1.0, rot=look_rotation(unit3(np.array([1, 1, 1], F32)))),
              light(abi.LIGHT_POINT, energy=2.0, rng_=10.0, pos=(2, 2, -3))]
    sd = SceneData([me], 1, lights, [[0, 1, 2]], name="uv_sphere")
    set_models_trs(sd, 0, [(0, 0, -5)], [(1, 1, 1)], quat_to_mat(random_quats(rng, 1)))
    sd.camera = camera(w=w, h=h, fov=75.0)
    return sd


def cubes_scene(seed=2, n=1000, w=1920, h=1080, nlights=8):
    """n unit cubes (shared mesh), positions U[-50,50]^3, random rotations, scales U[0.5,2];
    1920x1080 FOV 60 at the origin looking -Z; 8 coloured point lights, ambient 0.1."""
    rng = np.random.Generator(np.random.PCG64(seed))
    me = cube_mesh(1, 1, 1)
    pos = rng.uniform(-50, 50, (n, 3)).astype(F32)
    s = rng.uniform(0.5, 2.0, n).astype(F32)
    rot = quat_to_mat(random_quats(rng, n))
    lights = [light(abi.LIGHT_AMBIENT, energy=0.1)]
    for i in range(nlights):
        lights.append(light(abi.LIGHT_POINT, color=rng.uniform(0, 1, 3), energy=rng.uniform(0.5, 2.0),
                            rng_=rng.uniform(5, 20), pos=rng.uniform(-50, 50, 3)))
    sd = SceneData([me], n, lights, [list(range(len(lights)))], name="cubes")
    set_models_trs(sd, np.zeros(n, np.uint32), pos, np.repeat(s[:, None], 3, 1), rot)
    sd.camera = camera(w=w, h=h, fov=60.0)
    return sd


def terrain_scene(seed=3, n=1024, extent=200.0, w=3840, h=2160):
    """A value-noise grid of n x n vertices (4 octaves, amplitude 5) split into 4 quadrant models, each
    lit by its own LightGroup (ambient + directional + 4 of the 16 point lights + 2 box lights).
    3840x2160 FOV 70, camera 30 units up pitched -35 degrees, front-to-back sort."""
    rng = np.random.Generator(np.random.PCG64(seed))
    half = n // 2
    heights = lambda X, Z: 5.0 * value_noise(seed, X / 25.0, Z / 25.0, 4)
    step = extent / (n - 1)
    meshes = []
    for qz in range(2):
        for qx in range(2):
            i0, i1 = (0, half + 1) if qx == 0 else (half, n)
            j0, j1 = (0, half + 1) if qz == 0 else (half, n)
            me = grid_mesh(i1 - i0, j1 - j0, step * (i1 - i0 - 1), step * (j1 - j0 - 1), heights,
                           x0=-extent / 2 + i0 * step, z0=-extent / 2 + j0 * step)
            me.parts[0]["mat"] = default_material(sort_mode=abi.SORT_FRONT_TO_BACK)
            meshes.append(me)
    lights = [light(abi.LIGHT_AMBIENT, energy=0.15),
              light(abi.LIGHT_DIRECTIONAL, color=rng.uniform(0.5, 1, 3), energy=0.8,
                    rot=look_rotation(unit3(np.array([0.3, 1.0, 0.2], F32))))]
    for i in range(16):
        lights.append(light(abi.LIGHT_POINT, color=rng.uniform(0, 1, 3), energy=rng.uniform(0.5, 2.0),
                            rng_=rng.uniform(10, 40),
                            pos=(rng.uniform(-extent / 2, extent / 2), rng.uniform(2, 20), rng.uniform(-extent / 2, extent / 2))))
    cells = []
    for b in range(2):
        c = np.round(rng.uniform(-extent / 4, extent / 4, 3) * 4) / 4
        c[1] = 0.0
        vmin, vmax, cs = (c - 10).astype(F32), (c + 10).astype(F32), np.array([20, 20, 20], F32)
        counts = light_volume_counts(vmin, vmax, cs)
        first = len(cells)
        for _ in range(int(np.prod(counts))):
            cells.append(list(rng.uniform(0.2, 1.0, 3)) + [1.0])
        lights.append(light(abi.LIGHT_VOLUME, energy=1.0, vol=(vmin, vmax, cs, counts, first)))
    ambient, sun, points, boxes = 0, 1, list(range(2, 18)), [18, 19]
    lists = [list(range(len(lights)))]
    for g in range(4):
        lists.append([ambient, sun] + points[4 * g:4 * g + 4] + boxes)
    sd = SceneData(meshes, 4, lights, lists, cells=np.array(cells, F32), name="terrain")
    set_models_trs(sd, np.arange(4, dtype=np.uint32), np.zeros((4, 3)), np.ones((4, 3)), ident(4),
                   light_list=np.arange(1, 5))
    rot = rotate(1, 0, 0, deg2rad(-35.0))
    sd.camera = camera(pos=(0, 30, 0), rot=rot, w=w, h=h, fov=70.0)
    return sd


def batched_scene(seed=4, n=4096, vmin=24, vmax=65536, nlights=32, box=200.0, w=1920, h=1080, max_levels=6):
    """n models with log-uniform vertex counts in [vmin, vmax] (half noise-displaced grids of the exact
    count, half icospheres of the nearest level), transforms in [-box, box]^3, 32 point lights + ambient,
    a random LightGroup (ambient + random subset of the point lights) per model, random angular velocity
    steps for animation. Camera 1920x1080 at (0, 0, 1.5*box) looking -Z, far 3*box."""
    rng = np.random.Generator(np.random.PCG64(seed))
    targets = np.exp(rng.uniform(math.log(vmin), math.log(vmax), n)).astype(np.int64)
    ico = {}
    meshes, mesh_of = [], np.zeros(n, np.uint32)
    ico_levels = [icosphere(L) for L in range(max_levels + 1)]
    ico_counts = np.array([m.nverts for m in ico_levels])
    for i in range(n):
        if i % 2 == 0:
            lvl = int(np.argmin(np.abs(np.log(ico_counts) - math.log(targets[i]))))
            if lvl not in ico:
                ico[lvl] = len(meshes)
                meshes.append(ico_levels[lvl])
            mesh_of[i] = ico[lvl]
        else:
            side = max(5, int(round(math.sqrt(targets[i]))))
            nx, nz = side, max(5, int(targets[i] // side))
            sseed = int(rng.integers(1 << 30))
            me = grid_mesh(nx, nz, 4.0, 4.0 * nz / nx, lambda X, Z, s=sseed: 0.4 * value_noise(s, X, Z, 3),
                           x0=-2.0, z0=-2.0 * nz / nx)
            mesh_of[i] = len(meshes)
            meshes.append(me)
    pos = rng.uniform(-box, box, (n, 3)).astype(F32)
    scl = np.repeat(rng.uniform(1.0, 6.0, (n, 1)), 3, 1).astype(F32)
    rot = quat_to_mat(random_quats(rng, n))
    lights = [light(abi.LIGHT_AMBIENT, energy=0.1)]
    for _ in range(nlights):
        lights.append(light(abi.LIGHT_POINT, color=rng.uniform(0, 1, 3), energy=rng.uniform(0.5, 2.0),
                            rng_=rng.uniform(20, 80), pos=rng.uniform(-box, box, 3)))
    lists = [list(range(len(lights)))]
    groups = np.zeros(n, np.int32)
    for i in range(n):
        mask = rng.random(nlights) < 0.5
        lists.append([0] + [1 + k for k in range(nlights) if mask[k]])
        groups[i] = len(lists) - 1
    omega = rng.uniform(-1, 1, (n, 3)).astype(F32)
    dt = F32(1.0 / 60.0)
    steps = np.stack([rotate(*omega[i], float(np.linalg.norm(omega[i].astype(np.float64))) * dt) for i in range(n)])
    sd = SceneData(meshes, n, lights, lists, name="batched")
    set_models_trs(sd, mesh_of, pos, scl, rot, light_list=groups, step=steps)
    sd.camera = camera(pos=(0, 0, 1.5 * box), w=w, h=h, fov=60.0, near=0.1, far=3.0 * box)
    return sd


def _random_material(rng):
    """One mesh part's Material with every option drawn at random (material.go:40-120)."""
    alpha = 1.0 if rng.random() < 0.75 else float(rng.uniform(0.3, 0.9))
    tex = [0.0, 64.0, 256.0][int(rng.integers(3))]
    return default_material(
        color=(float(rng.uniform(0.5, 1)), float(rng.uniform(0.5, 1)), float(rng.uniform(0.5, 1)), alpha),
        tex_w=tex, tex_h=tex / 2, present=int(rng.random() < 0.95), backface_culling=int(rng.random() < 0.8),
        sort_mode=int(rng.integers(3)), lighting_mode=int(rng.integers(3)), lv_shading_mode=int(rng.integers(4)),
        shadeless=int(rng.random() < 0.1), visible=int(rng.random() < 0.95),
        transparency_mode=[abi.TRANSPARENCY_AUTO, abi.TRANSPARENCY_AUTO, abi.TRANSPARENCY_OPAQUE,
                           abi.TRANSPARENCY_ALPHA_CLIP, abi.TRANSPARENCY_TRANSPARENT][int(rng.integers(5))],
        blend_source_over=int(rng.random() < 0.9), render_order=[0, 0, 0, 1, -1][int(rng.integers(5))])


def feature_scene(seed=5, n=48, w=1280, h=720):
    """Small meshes under every material, model and light option of the vertex stage.

    Meshes: icospheres (flat normals, vertex colours) and noise grids split into 1-3 parts, cubes and a UV
    sphere without a colour channel; each mesh copy gets random part materials (sort mode, backface culling,
    lighting mode, light-volume shading mode, shadeless, visibility, transparency mode, additive blending,
    render order, material alpha, texture size, nil material). Models: random transforms in front of the
    camera plus a few behind it and beyond the far plane, random tint and alpha (one fully transparent),
    invisible and shadeless models, frustum culling switched off on some. Lights: ambient, three point, two
    directional and two volume lights; the scene list plus three LightGroups.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    bases = []
    for lvl in (1, 2):
        me = icosphere(lvl)
        me.colors = rng.uniform(0.4, 1.0, (me.nverts, 4)).astype(F32)
        bases.append(me)
    for k in range(2):
        sseed = int(rng.integers(1 << 30))
        me = grid_mesh(14, 10, 4.0, 3.0, lambda X, Z, s=sseed: 0.5 * value_noise(s, X, Z, 2), x0=-2.0, z0=-1.5)
        me.colors = rng.uniform(0.4, 1.0, (me.nverts, 4)).astype(F32)
        bases.append(me)
    bases.append(cube_mesh(1.5, 1.0, 2.0))
    bases.append(uv_sphere(16, 8, 1.2))
    meshes = []
    for k in range(16):
        b = bases[k % len(bases)]
        T = b.ntris
        nparts = 1 if T < 24 else int(rng.integers(1, 4))
        cuts = sorted(set([0, T] + [int(c) for c in rng.integers(1, T, nparts - 1)]))
        parts = [dict(tri_start=cuts[i], tri_count=cuts[i + 1] - cuts[i], mat=_random_material(rng))
                 for i in range(len(cuts) - 1)]
        meshes.append(MeshData(b.positions, b.normals, b.uvs, b.indices, colors=b.colors, parts=parts))
    pos = np.stack([rng.uniform(-14, 14, n), rng.uniform(-8, 8, n), rng.uniform(-45, -4, n)], 1).astype(F32)
    pos[0] = (0, 0, 150)    # far behind the camera: outside the frustum sphere
    pos[1] = (2, 0, -90)    # beyond the far plane, frustum culling off below
    scl = np.repeat(rng.uniform(0.5, 3.0, (n, 1)), 3, 1).astype(F32)
    scl[2] = (1.0, 2.0, 0.5)  # non-uniform scale
    rot = quat_to_mat(random_quats(rng, n))
    cells = []
    lights = [light(abi.LIGHT_AMBIENT, color=(0.9, 0.95, 1.0), energy=0.25)]
    for _ in range(3):
        lights.append(light(abi.LIGHT_POINT, color=rng.uniform(0.3, 1, 3), energy=rng.uniform(1, 4),
                            rng_=rng.uniform(8, 30), pos=(rng.uniform(-12, 12), rng.uniform(-6, 6), rng.uniform(-40, -5))))
    for d in ([0.3, 1.0, 0.2], [-0.7, -0.2, 0.6]):
        lights.append(light(abi.LIGHT_DIRECTIONAL, color=rng.uniform(0.5, 1, 3), energy=rng.uniform(0.4, 1.2),
                            rot=look_rotation(unit3(np.array(d, F32)))))
    for c in ((-6.0, 0.0, -20.0), (7.0, 2.0, -30.0)):
        c = np.asarray(c, F32)
        vmin, vmax, cs = c - F32(9), c + F32(9), np.array([4.5, 6.0, 3.0], F32)
        counts = light_volume_counts(vmin, vmax, cs)
        first = len(cells)
        for _ in range(int(np.prod(counts))):
            cells.append(list(rng.uniform(0.1, 1.0, 3)) + [1.0])
        lights.append(light(abi.LIGHT_VOLUME, energy=float(rng.uniform(0.5, 1.5)), vol=(vmin, vmax, cs, counts, first)))
    lists = [list(range(len(lights))), [0, 1, 4], [0, 2, 3, 6], [5, 7, 1]]
    groups = np.where(rng.random(n) < 0.5, -1, rng.integers(1, 4, n)).astype(np.int32)
    mesh_of = rng.integers(0, len(meshes), n).astype(np.uint32)
    colors = np.ones((n, 4), F32)
    tint = rng.random(n) < 0.3
    colors[tint, :3] = rng.uniform(0.3, 1.0, (int(tint.sum()), 3))
    half = rng.random(n) < 0.15
    colors[half, 3] = 0.5
    colors[3, 3] = 0.0      # fully transparent model: skipped
    sd = SceneData(meshes, n, lights, lists, cells=np.array(cells, F32), name=f"features{seed}")
    set_models_trs(sd, mesh_of, pos, scl, rot, light_list=groups)
    sd.mv["color"] = colors
    sd.mv["frustum_culling"] = (rng.random(n) < 0.85).astype(np.int32)
    sd.mv["frustum_culling"][0] = 1  # culled by SphereInFrustum
    sd.mv["frustum_culling"][1] = 0  # reaches the per-triangle far-plane test
    sd.mv["visible"][:2] = 1
    sd.mv["visible"] = (rng.random(n) < 0.95).astype(np.int32)
    sd.mv["shadeless"] = (rng.random(n) < 0.1).astype(np.int32)
    sd.camera = feature_camera("persp", w, h)
    return sd


def tube_mesh(rings=12, segments=10, height=3.0, radius=0.35):
    """An open cylinder along +Y: (rings + 1) x segments vertices, smooth radial normals."""
    r = np.arange(rings + 1)[:, None]
    sg = np.arange(segments)[None, :]
    ph = 2 * np.pi * sg / segments + 0 * r
    y = height * r / rings + 0 * sg
    pos = np.stack([radius * np.cos(ph), y, radius * np.sin(ph)], -1).reshape(-1, 3).astype(F32)
    nrm = np.stack([np.cos(ph), 0 * ph, np.sin(ph)], -1).reshape(-1, 3).astype(F32)
    uv = np.stack([sg / segments + 0 * r, r / rings + 0 * sg], -1).reshape(-1, 2).astype(F32)
    q = (np.arange(rings)[:, None] * segments + np.arange(segments)[None, :]).reshape(-1)
    nxt = (q // segments) * segments + (q + 1) % segments
    idx = np.stack([q, nxt, q + segments, nxt, nxt + segments, q + segments], 1).reshape(-1, 3).astype(np.uint32)
    idx = _orient_outward(pos, idx, center=None)
    return MeshData(pos, nrm, uv, idx)


def tube_skin(me, rng, nbones=4, height=3.0):
    """Joints and weights of a tube along Y: each vertex blends the two nearest of `nbones` bones
    spaced along the tube (exact 1.0 weights on the bone heights), unused slots hold other joints with
    weight 0, and a few vertices carry a 1.0 weight after a partial one (Model.skinVertex stops there)."""
    f = me.positions[:, 1].astype(np.float64) / height * (nbones - 1)
    i0 = np.clip(np.floor(f), 0, nbones - 2).astype(np.uint32)
    t = (f - i0).astype(F32)
    V = me.nverts
    joints = np.zeros((V, 4), np.uint32)
    weights = np.zeros((V, 4), F32)
    joints[:, 0], joints[:, 1] = i0, i0 + 1
    weights[:, 0], weights[:, 1] = F32(1) - t, t
    joints[:, 2:] = rng.integers(0, nbones, (V, 2))
    weights[t == 0, :] = (1, 0, 0, 0)
    weights[t == 1, :] = (0, 1, 0, 0)
    odd = rng.choice(V, max(1, V // 12), replace=False)
    weights[odd] = (0.25, 1.0, 0.5, 0.0)
    return joints, weights


def tube_bones(rng, n, pos, nbones=4, height=3.0, bend=0.5):
    """Per model a chain of bone influence matrices bending a tube at `pos` (row-vector TRS)."""
    out = []
    for k in range(n):
        for b in range(nbones):
            ang = [float(rng.uniform(-bend, bend)) * b / max(nbones - 1, 1) for _ in range(2)]
            rot = mult(rotate(1, 0, 0, ang[0]), rotate(0, 0, 1, ang[1]))
            off = np.asarray(pos[k], F32) + np.array([0.3 * ang[1] * b, 0.0, 0.3 * ang[0] * b], F32)
            s = F32(rng.uniform(0.8, 1.2))
            out.append(trs(off.reshape(1, 3), np.full((1, 3), s, F32), rot.reshape(1, 4, 4))[0])
    return np.asarray(out, F32).reshape(-1, 4, 4)


def skinned_scene(seed=7, n=28, w=1280, h=720):
    """Skinned and shape-keyed meshes under the feature scene's lights and random materials.

    Meshes: a skinned tube (two copies with different part materials), a skinned tube that also has a
    shape key, a UV sphere with two shape keys and a cube. Models: skinned tubes each bent by its own bone
    chain (one behind the camera, culled on its model position), tubes drawn unskinned, shape-keyed spheres
    under random transforms and a few cubes. Lights, light volumes and light lists as in feature_scene.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    base = feature_scene(seed, n=4)
    nb = 4
    tubes = []
    for k in range(3):
        t = tube_mesh()
        T = t.ntris
        cuts = sorted(set([0, T] + [int(c) for c in rng.integers(1, T, 2)]))
        t.parts = [dict(tri_start=cuts[i], tri_count=cuts[i + 1] - cuts[i], mat=_random_material(rng))
                   for i in range(len(cuts) - 1)]
        t.joints, t.weights = tube_skin(t, rng, nb)
        t.colors = rng.uniform(0.4, 1.0, (t.nverts, 4)).astype(F32) if k != 1 else None
        tubes.append(t)
    pinch = np.zeros((1, tubes[2].nverts, 3), F32)
    pinch[0] = -0.3 * tubes[2].positions * np.array([1, 0, 1], F32) * np.sin(
        tubes[2].positions[:, 1:2] * F32(np.pi / 3)).astype(F32)
    tubes[2].shape_positions = pinch
    tubes[2].shape_normals = rng.uniform(-0.2, 0.2, pinch.shape).astype(F32)
    tubes[2].shape_weights = np.array([0.6], F32)
    sph = uv_sphere(16, 8, 1.2)
    sph.parts = [dict(tri_start=0, tri_count=sph.ntris, mat=_random_material(rng))]
    bulge = (sph.normals * rng.uniform(0.0, 0.4, (sph.nverts, 1))).astype(F32)
    sph.shape_positions = np.stack([bulge, rng.uniform(-0.15, 0.15, bulge.shape).astype(F32)])
    sph.shape_normals = rng.uniform(-0.3, 0.3, (2, sph.nverts, 3)).astype(F32)
    sph.shape_weights = np.array([0.7, -0.35], F32)
    cube = cube_mesh(1.0, 1.0, 1.0)
    cube.parts = [dict(tri_start=0, tri_count=cube.ntris, mat=_random_material(rng))]
    meshes = tubes + [sph, cube]
    nskin = n // 2
    pos = np.stack([rng.uniform(-12, 12, n), rng.uniform(-6, 4, n), rng.uniform(-34, -6, n)], 1).astype(F32)
    pos[1] = (0, 0, 150)  # skinned, behind the camera: culled on the model position
    mesh_of = np.empty(n, np.uint32)
    mesh_of[:nskin] = rng.integers(0, 3, nskin)
    rest = n - nskin
    mesh_of[nskin:] = rng.choice([0, 2, 3, 3, 3, 4], rest)
    scl = np.repeat(rng.uniform(0.6, 2.0, (n, 1)), 3, 1).astype(F32)
    rot = quat_to_mat(random_quats(rng, n))
    sd = SceneData(meshes, n, [base.lights[i] for i in range(base.nlights)], base.lists,
                   cells=base.cells[:base.ncells] if base.ncells else None, name=f"skinned{seed}")
    set_models_trs(sd, mesh_of, pos, scl, rot,
                   light_list=np.where(rng.random(n) < 0.5, -1, rng.integers(1, 4, n)).astype(np.int32))
    sd.mv["skinned"][:nskin] = 1
    sd.mv["bone_first"][:nskin] = np.arange(nskin, dtype=np.uint32) * nb
    sd.mv["frustum_culling"] = (rng.random(n) < 0.85).astype(np.int32)
    sd.mv["frustum_culling"][1] = 1
    sd.mv["shadeless"] = (rng.random(n) < 0.08).astype(np.int32)
    tint = rng.random(n) < 0.3
    sd.mv["color"][tint, :3] = rng.uniform(0.3, 1.0, (int(tint.sum()), 3))
    sd.bones = tube_bones(rng, nskin, pos[:nskin], nb)
    sd.camera = feature_camera("persp", w, h)
    return sd


def quad_mesh(w=1.0, h=1.0):
    """A w x h quad in the XY plane facing +Z (two triangles)."""
    w2, h2 = F32(w) / F32(2), F32(h) / F32(2)
    pos = np.array([(-w2, -h2, 0), (w2, -h2, 0), (w2, h2, 0), (-w2, h2, 0)], F32)
    nrm = np.tile(np.array([0, 0, 1], F32), (4, 1))
    uv = np.array([(0, 0), (1, 0), (1, 1), (0, 1)], F32)
    return MeshData(pos, nrm, uv, np.array([(0, 1, 2), (0, 2, 3)], np.uint32))


BILLBOARD_OPTIONS = [  # (locks, up, depth mode)
    ((0, 0, 0), 0, 0), ((0, 1, 0), 0, 0), ((1, 0, 0), 0, 0), ((0, 0, 1), 0, 0), ((0, 0, 0), 1, 0),
    ((0, 0, 0), 0, 1), ((1, 1, 0), 1, 1), ((0, 1, 1), 0, 1)]


def billboard_scene(seed=9, n=40, w=1280, h=720):
    """Billboarded parts under every lock, up direction and depth mode (Material.Billboard*),
    next to plain parts of the same meshes, under the feature scene's lights.

    Meshes: quads (two triangles, one part) and icospheres with two parts, one billboarded and one
    not; each copy takes one option set of BILLBOARD_OPTIONS on top of a random material. Models: random
    transforms in front of the camera, one directly below a camera at (0, 10, 0) (the LookAt's
    degenerate-up branch for that camera) and a skinned tube with a billboard material (not turned).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    base = feature_scene(seed, n=4)
    meshes = []
    for k, (locks, up, depth) in enumerate(BILLBOARD_OPTIONS):
        bb = dict(billboard=1, billboard_lock=locks, billboard_up=up, billboard_depth=depth)
        q = quad_mesh(float(rng.uniform(0.8, 2.5)), float(rng.uniform(0.8, 2.5)))
        q.parts = [dict(tri_start=0, tri_count=2, mat={**_random_material(rng), **bb, "present": 1, "visible": 1})]
        q.colors = rng.uniform(0.4, 1.0, (4, 4)).astype(F32) if k % 2 else None
        meshes.append(q)
        ico = icosphere(1)
        T = ico.ntris
        cut = int(rng.integers(8, T - 8))
        ico.parts = [dict(tri_start=0, tri_count=cut, mat={**_random_material(rng), **bb, "present": 1, "visible": 1}),
                     dict(tri_start=cut, tri_count=T - cut, mat=_random_material(rng))]
        meshes.append(ico)
    tube = tube_mesh(rings=4, segments=6)
    tube.joints, tube.weights = tube_skin(tube, rng, 4)
    tube.parts = [dict(tri_start=0, tri_count=tube.ntris,
                       mat=default_material(billboard=1, billboard_depth=1, backface_culling=0))]
    meshes.append(tube)
    nb = len(meshes) - 1
    pos = np.stack([rng.uniform(-12, 12, n), rng.uniform(-6, 6, n), rng.uniform(-35, -5, n)], 1).astype(F32)
    pos[0] = (0.0, 0.0, 0.0)   # below a camera at (0, 10, 0) looking down
    pos[1] = (0.5, 1.0, -12.0)
    mesh_of = np.concatenate([np.arange(nb), rng.integers(0, nb, n - nb - 1), [nb]]).astype(np.uint32)
    scl = np.repeat(rng.uniform(0.6, 2.0, (n, 1)), 3, 1).astype(F32)
    rot = quat_to_mat(random_quats(rng, n))
    rot[0] = ident()
    scl[0] = 3.0
    sd = SceneData(meshes, n, [base.lights[i] for i in range(base.nlights)], base.lists,
                   cells=base.cells[:base.ncells] if base.ncells else None, name=f"billboards{seed}")
    set_models_trs(sd, mesh_of, pos, scl, rot,
                   light_list=np.where(rng.random(n) < 0.5, -1, rng.integers(1, 4, n)).astype(np.int32))
    sd.mv["frustum_culling"] = (rng.random(n) < 0.7).astype(np.int32)
    sd.mv["frustum_culling"][0] = 0
    sd.mv["skinned"][n - 1] = 1
    sd.bones = tube_bones(rng, 1, pos[n - 1:], 4)
    sd.camera = feature_camera("persp", w, h)
    return sd


SUBDIVISION_LEVELS = [(36.0, 0.6), (144.0, 1.2), (576.0, 3.0)]  # (DistanceSquared, MaximumTriangleSize)


def subdivision_scene(seed=10, n=24, w=1280, h=720, max_subdivisions=3):
    """Auto-subdivided meshes (Mesh.SetAutoSubdivide) seen from 2 to 40 units away, so each draws
    its base triangles or one of three subdivision levels, next to the same meshes unsubdivided.

    Meshes: a coarse noise grid (large triangles), an icosahedron scaled up, a cube with vertex colours
    and two parts, each once with auto-subdivision on and once off. Levels: SUBDIVISION_LEVELS; some
    triangles are shorter than the smallest size (never subdivided) and some stop subdividing before
    the last level (empty deeper lists).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    base = feature_scene(seed, n=4)
    meshes = []
    sseed = int(rng.integers(1 << 30))
    grid = grid_mesh(6, 5, 6.0, 5.0, lambda X, Z, s=sseed: 0.8 * value_noise(s, X, Z, 2), x0=-3.0, z0=-2.5)
    grid.colors = rng.uniform(0.4, 1.0, (grid.nverts, 4)).astype(F32)
    ico = icosphere(0)
    ico.positions = (ico.positions * F32(2.5)).astype(F32)
    cube = cube_mesh(3.0, 0.5, 2.0)
    cube.colors = rng.uniform(0.4, 1.0, (cube.nverts, 4)).astype(F32)
    for b in (grid, ico, cube):
        T = b.ntris
        cut = int(rng.integers(1, T))
        for sub in (1, 0):
            m = MeshData(b.positions, b.normals, b.uvs, b.indices, colors=b.colors,
                         parts=[dict(tri_start=0, tri_count=cut, mat=_random_material(rng)),
                                dict(tri_start=cut, tri_count=T - cut, mat=_random_material(rng))])
            for p in m.parts:
                p["mat"].update(present=1, visible=1)
            m.auto_subdivide = sub
            meshes.append(m)
    dist = rng.uniform(2.0, 40.0, n)
    dirs = unit3(np.stack([rng.uniform(-0.5, 0.5, n), rng.uniform(-0.3, 0.3, n), -np.ones(n)], 1).astype(F32))
    pos = (dirs * dist[:, None].astype(F32)).astype(F32)
    mesh_of = rng.integers(0, len(meshes), n).astype(np.uint32)
    mesh_of[:len(meshes)] = np.arange(len(meshes))
    scl = np.repeat(rng.uniform(0.7, 1.5, (n, 1)), 3, 1).astype(F32)
    rot = quat_to_mat(random_quats(rng, n))
    sd = SceneData(meshes, n, [base.lights[i] for i in range(base.nlights)], base.lists,
                   cells=base.cells[:base.ncells] if base.ncells else None, name=f"subdivision{seed}")
    set_models_trs(sd, mesh_of, pos, scl, rot,
                   light_list=np.where(rng.random(n) < 0.5, -1, rng.integers(1, 4, n)).astype(np.int32))
    sd.mv["frustum_culling"] = (rng.random(n) < 0.7).astype(np.int32)
    sd.subdivision_levels = np.array(SUBDIVISION_LEVELS, F32)
    sd.max_subdivisions = max_subdivisions
    sd.camera = feature_camera("persp", w, h)
    return sd


TEXTURE_SIZES = [(64, 32), (16, 16), (128, 64)]


def raster_textures(seed=0, holes=True):
    """Premultiplied RGBA8 textures of TEXTURE_SIZES: random colours, and with `holes` a band of
    texels at or below the alpha clip's 0.8 (alpha 0 or 204) and a band just above it (230)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for w, h in TEXTURE_SIZES:
        a = np.full((h, w), 255, np.uint8)
        if holes:
            a[:, : w // 4] = 0
            a[: h // 4, :] = 204
            a[h // 2: h // 2 + h // 8, :] = 230
        rgb = np.floor(rng.integers(0, 256, (h, w, 3)) * (a[..., None] / 255.0)).astype(np.uint8)
        out.append(np.ascontiguousarray(np.concatenate([rgb, a[..., None]], -1)))
    return out


def texture_materials(sd, seed):
    """Textures a scene's materials in place: each names one of raster_textures (or the white
    default) with its size, a random filter, UV or screen mapping with a random screen multiplier,
    and alpha clip on some. Returns the scene."""
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    for m in sd.meshes:
        for p in m.parts:
            mat = p["mat"]
            t = int(rng.integers(len(TEXTURE_SIZES) + 1))
            tw, th = TEXTURE_SIZES[t - 1] if t else (0, 0)
            mat.update(texture=t, tex_w=float(tw), tex_h=float(th), texture_filter=int(rng.random() < 0.5),
                       texture_map_mode=int(rng.random() < 0.2),
                       texture_map_scale=[(1.0, 1.0), (0.5, 0.25), (2.0, 1.5)][int(rng.integers(3))])
            if rng.random() < 0.3:
                mat["transparency_mode"] = abi.TRANSPARENCY_ALPHA_CLIP
    sd.name = f"{sd.name}_textured"
    return sd


FRAME_VARIANTS = ("shape_keys", "skinned", "billboard", "subdivision", "batched")


def frame_variant(kind, seed=4, n=4096):
    """The benchmark frame (batched_scene) with one vertex-stage feature switched on at scale:
    'shape_keys' (two keys on every mesh), 'skinned' (every model skinned by a four-bone chain
    bending it about its own axis), 'billboard' (every material billboarded, camera-Y up),
    'subdivision' (the icospheres of up to 320 triangles auto-subdivided up to twice within 250
    units) and 'batched' (the noise grids drawn in the dynamic batches of 16 icosphere owners)."""
    sd = batched_scene(seed, n=n)
    rng = np.random.Generator(np.random.PCG64(seed + 77))
    if kind == "shape_keys":
        for m in sd.meshes:
            bulge = (m.normals * rng.uniform(0.0, 0.2, (m.nverts, 1))).astype(F32)
            m.shape_positions = np.stack([bulge, rng.uniform(-0.05, 0.05, bulge.shape).astype(F32)])
            m.shape_normals = rng.uniform(-0.1, 0.1, (2, m.nverts, 3)).astype(F32)
            m.shape_weights = np.array([0.6, -0.3], F32)
    elif kind == "skinned":
        nb = 4
        for m in sd.meshes:
            y = m.positions[:, 1].astype(np.float64)
            f = (y - y.min()) / max(y.max() - y.min(), 1e-6) * (nb - 1)
            i0 = np.clip(np.floor(f), 0, nb - 2).astype(np.uint32)
            t = (f - i0).astype(F32)
            m.joints = np.zeros((m.nverts, 4), np.uint32)
            m.weights = np.zeros((m.nverts, 4), F32)
            m.joints[:, 0], m.joints[:, 1] = i0, i0 + 1
            m.weights[:, 0], m.weights[:, 1] = F32(1) - t, t
        M = sd.mv["transform"].reshape(n, 4, 4)
        bones = np.empty((n * nb, 4, 4), F32)
        for k in range(n):
            for b in range(nb):
                bend = mult(rotate(1, 0, 0, 0.15 * b), rotate(0, 0, 1, -0.1 * b))
                bones[k * nb + b] = mult(bend, M[k])
        sd.mv["skinned"] = 1
        sd.mv["bone_first"] = np.arange(n, dtype=np.uint32) * nb
        sd.bones = bones
    elif kind == "billboard":
        for m in sd.meshes:
            for p in m.parts:
                p["mat"].update(billboard=1, billboard_lock=(0, 0, 0), billboard_up=abi.BILLBOARD_UP_CAMERA_Y,
                                billboard_depth=abi.DEPTH_DEFAULT)
    elif kind == "subdivision":
        for m in sd.meshes:
            if m.ntris <= 320:
                m.auto_subdivide = 1
        sd.subdivision_levels = np.array([(250.0 * 250.0, 0.3)], F32)  # model-space triangle size
        sd.max_subdivisions = 2
    elif kind == "batched":
        owners = np.arange(0, 32, 2)  # icospheres (even models)
        members = np.arange(1, n, 2)  # noise grids
        sd.mv["batched"][members] = 1
        sd.mv["batch_owner"][members] = owners[rng.integers(0, len(owners), len(members))]
        sd.mv["batch_part"][members] = 0
    else:
        raise ValueError(kind)
    sd.name = f"{sd.name}_{kind}"
    return sd


def textured_scene(seed=21, n=48, w=1280, h=720):
    """The feature scene with textured materials (texture_materials)."""
    return texture_materials(feature_scene(seed, n=n, w=w, h=h), seed)


def batch_scene(seed=11, n=72, w=1280, h=720):
    """Dynamic batches (Model.DynamicBatchAdd): three owners, two of them batching under two
    of their mesh parts, with members from the feature meshes scattered in front of the camera
    (some invisible, some behind the camera with frustum culling, one half-transparent so one
    batch goes to the transparent pass), next to unbatched models of the same meshes.
    Owner 2 is itself a member of owner 0's batch (its own batch is never drawn)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    base = feature_scene(seed, n=8)
    owner_mesh = cube_mesh(1.0, 1.0, 1.0)
    owner_mesh.parts = [dict(tri_start=0, tri_count=6, mat=_random_material(rng)),
                        dict(tri_start=6, tri_count=6, mat=_random_material(rng))]
    for p in owner_mesh.parts:
        p["mat"].update(present=1, visible=1, transparency_mode=abi.TRANSPARENCY_OPAQUE, render_order=0)
    meshes = list(base.meshes[:6]) + [owner_mesh]
    om = len(meshes) - 1
    sd = SceneData(meshes, n, [base.lights[i] for i in range(base.nlights)], base.lists,
                   cells=base.cells[:base.ncells] if base.ncells else None, name=f"batches{seed}")
    pos = np.stack([rng.uniform(-14, 14, n), rng.uniform(-8, 8, n), rng.uniform(-45, -4, n)], 1).astype(F32)
    mesh_of = rng.integers(0, 6, n).astype(np.uint32)
    mesh_of[:3] = om
    scl = np.repeat(rng.uniform(0.5, 2.0, (n, 1)), 3, 1).astype(F32)
    rot = quat_to_mat(random_quats(rng, n))
    set_models_trs(sd, mesh_of, pos, scl, rot,
                   light_list=np.where(rng.random(n) < 0.5, -1, rng.integers(1, 4, n)).astype(np.int32))
    mv = sd.mv
    mv["frustum_culling"] = 1
    members = np.arange(3, n - 10)
    mv["batched"][members] = 1
    mv["batch_owner"][members] = rng.integers(0, 2, len(members))
    mv["batch_part"][members] = rng.integers(0, 2, len(members))
    mv["batched"][2], mv["batch_owner"][2], mv["batch_part"][2] = 1, 0, 1   # a nested owner
    mv["batched"][n - 12], mv["batch_owner"][n - 12], mv["batch_part"][n - 12] = 1, 2, 0
    mv["visible"][[5, 9]] = 0
    mv["position"][7] = (0.0, 0.0, 60.0)  # behind the camera: culled inside its batch
    mv["color"][11] = (1.0, 1.0, 1.0, 0.5)  # makes its owner's later batch parts transparent
    M = trs(mv["position"], mv["scale"], mv["rotation"].reshape(n, 4, 4))
    mv["transform"] = M.reshape(n, 16)
    sd.camera = feature_camera("persp", w, h)
    return sd


def down_camera(w=1280, h=720):
    """A camera at (0, 10, 0) looking straight down -Y."""
    return camera(pos=(0.0, 10.0, 0.0), rot=rotate(1, 0, 0, deg2rad(-90.0)), w=w, h=h, fov=70.0, near=0.1, far=60.0)


def nested_light_scene(seed=5, n=48, w=1280, h=720):
    """The feature scene with LightVolumeCell.useLights: about 70 % of the light-volume cells
    use one to three of the scene's ambient, point and directional lights (the lights may also be
    in the light lists)."""
    sd = feature_scene(seed, n, w, h)
    rng = np.random.Generator(np.random.PCG64([seed, 77]))
    usable = [i for i in range(sd.nlights) if sd.lights[i].type != abi.LIGHT_VOLUME]
    sd.cell_uses = [list(rng.choice(usable, int(rng.integers(1, 4)), replace=False)) if rng.random() < 0.7 else []
                    for _ in range(sd.ncells)]
    sd.name = f"nested{seed}"
    return sd


FEATURE_CAMERAS = ["persp", "ortho", "unlit", "fog_add", "fog_sub", "fog_overwrite", "corrected", "tilted"]


def feature_camera(variant, w=1280, h=720):
    """Camera options of camera.go: perspective / orthographic, lighting off, fog modes with depth
    rendering off, perspective-corrected UVs, a rotated and moved camera."""
    kw = dict(w=w, h=h, fov=65.0, near=0.1, far=60.0)
    if variant == "ortho":
        kw.update(perspective=0, ortho_scale=40.0)
    elif variant == "unlit":
        kw.update(lighting_on=0)
    elif variant.startswith("fog_"):
        kw.update(render_depth=0, fog_on=1,
                  fog_mode={"fog_add": abi.FOG_ADD, "fog_sub": abi.FOG_SUB, "fog_overwrite": abi.FOG_OVERWRITE}[variant])
    elif variant == "tilted":
        kw.update(pos=(3.0, 4.0, 2.0), rot=mult(rotate(1, 0, 0, deg2rad(-12.0)), rotate(0, 1, 0, deg2rad(8.0))))
    c = camera(**kw)
    if variant.startswith("fog_"):
        c.fog_range[:] = [0.15, 0.85]
        c.fog_color[:] = [0.4, 0.5, 0.9, 1.0]
    if variant == "corrected":
        c.perspective_corrected = 1
    return c


def corrected_camera(variant, w=1280, h=720):
    """feature_camera(variant) with Camera.PerspectiveCorrectedTextureMapping on."""
    c = feature_camera(variant, w, h)
    c.perspective_corrected = 1
    return c


def small_variant(kind, seed):
    """Reduced-size versions of the workloads for oracle comparisons."""
    if kind == "sphere":
        return uv_sphere_scene(seed)
    if kind == "cubes":
        return cubes_scene(seed, n=200)
    if kind == "terrain":
        return terrain_scene(seed, n=96, extent=60.0, w=1280, h=720)
    if kind == "batched":
        return batched_scene(seed, n=48, vmin=24, vmax=6000, nlights=8, box=40.0, max_levels=4)
    raise ValueError(kind)


def subset(sd, models):
    """A SceneData with only the given models (meshes, lights and light lists shared)."""
    models = np.asarray(models, np.int64)
    out = SceneData(sd.meshes, len(models), [sd.lights[i] for i in range(sd.nlights)], sd.lists,
                    cells=sd.cells[:sd.ncells] if sd.ncells else None, name=sd.name + f"[{len(models)}]")
    out.mv[:] = sd.mv[models]
    out.camera = sd.camera
    out.bones = sd.bones
    out.subdivision_levels = sd.subdivision_levels
    out.max_subdivisions = sd.max_subdivisions
    out.cell_uses = sd.cell_uses
    return out
