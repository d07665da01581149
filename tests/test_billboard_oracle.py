"""The oracle's billboarding (ProcessVertices with Material.BillboardEnabled,
model.go:634-703) against a float32 numpy restatement: a billboarded part
emits the corners of the same part under a plain model whose transform is the
billboarded matrix, and with DepthModeUnbillboarded its depth is that of the
unturned model."""
import numpy as np
import pytest

from oracle import pyoracle
from tetra3d_gb300 import abi, scenes

F32 = np.float32


def _unit(v):
    v = np.asarray(v, F32)
    ln = F32(np.sqrt(np.float64(F32(F32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))))
    if ln < F32(1e-8) or ln == F32(1):
        return v.copy()
    return np.array([v[0] / ln, v[1] / ln, v[2] / ln], F32)


def _cross(a, b):
    return np.array([a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]], F32)


def _equals(a, b):
    return not np.any(np.abs((np.asarray(a, F32) - np.asarray(b, F32)).astype(F32)) > F32(1e-4))


def _look_at(frm, to, up):
    if _equals(frm, to):
        return scenes.ident()
    z = _unit((np.asarray(to, F32) - np.asarray(frm, F32)).astype(F32))
    up = _unit(up)
    if _equals(z, up) or _equals(z, -up):
        up = np.array([1, 0, 0], F32) if not _equals(up, [1, 0, 0]) else np.array([0, 0, 1], F32)
    x = _unit(_cross(up, z))
    y = _cross(z, x)
    m = scenes.ident()
    m[0, :3], m[1, :3], m[2, :3] = x, y, z
    return m


def _unit_row(m, i):
    m[i, :3] = _unit(m[i, :3])


def _decompose(M):
    rot = scenes.ident()
    for i in range(3):
        rot[i, :3] = _unit(M[i, :3])
        rot[i, 3] = M[i, 3]
    inn = scenes.mult(M, rot.T.copy())
    s = np.array([np.sqrt(np.float64(F32(F32(inn[i, 0] * inn[i, 0] + inn[i, 1] * inn[i, 1]) + inn[i, 2] * inn[i, 2])))
                  for i in range(3)], F32)
    return M[3, :3].copy(), s, rot


def billboard_base(M, cam_pos, up, locks):
    L = _look_at(M[3, :3], cam_pos, up)
    if locks[0]:
        L[0] = (1, 0, 0, 0); L[1, 0] = 0; _unit_row(L, 1); L[2, 0] = 0; _unit_row(L, 2)
    if locks[1]:
        L[1] = (0, 1, 0, 0); L[0, 1] = 0; _unit_row(L, 0); L[2, 1] = 0; _unit_row(L, 2)
    if locks[2]:
        L[2] = (0, 0, 1, 0); L[0, 2] = 0; _unit_row(L, 0); L[1, 2] = 0; _unit_row(L, 1)
    p, s, r = _decompose(M)
    base = scenes.mult(scenes.mult(r, scenes.scale_m(*s)), L)
    base[3] = (p[0], p[1], p[2], 1)
    return base


def _scene(mat, transform):
    q = scenes.quad_mesh(1.5, 1.0)
    q.parts = [dict(tri_start=0, tri_count=2, mat=mat)]
    sd = scenes.SceneData([q], 1, [], [[]], name="bb")
    scenes.set_models_trs(sd, [0], np.zeros((1, 3), F32), np.ones((1, 3), F32), scenes.ident(1), frustum=0)
    sd.mv["use_trs"] = 0
    sd.mv["transform"] = np.asarray(transform, F32).reshape(1, 16)
    return sd


def _by_tri(f):
    order = np.argsort(f.tri_index, kind="stable")
    return f.tri_index[order], f.xyuv[order], f.depth[order]


@pytest.mark.parametrize("opt", range(len(scenes.BILLBOARD_OPTIONS)))
@pytest.mark.parametrize("cam_kind", ["persp", "tilted", "down"])
def test_billboard_matches_numpy_restatement(opt, cam_kind):
    locks, up_mode, _ = scenes.BILLBOARD_OPTIONS[opt]
    cam = scenes.down_camera() if cam_kind == "down" else scenes.feature_camera(cam_kind)
    cam.fog_on = 0
    rng = np.random.default_rng(opt)
    rot = scenes.quat_to_mat(scenes.random_quats(rng, 1))[0] if opt % 2 else scenes.ident()
    pos = np.array([0.0, 0.0, 0.0] if cam_kind == "down" else [1.5, -0.5, -9.0], F32)
    M = scenes.trs(pos, np.array([1.3, 0.8, 1.1], F32), rot)[0]
    mat = scenes.default_material(shadeless=1, backface_culling=0, billboard=1, billboard_lock=locks,
                                  billboard_up=up_mode, billboard_depth=abi.DEPTH_DEFAULT)
    cam_pos = np.asarray(cam.transform[:], F32).reshape(4, 4)[3, :3]
    cam_up = _unit(np.asarray(cam.world_rotation[:], F32).reshape(4, 4)[1, :3])
    up = cam_up if up_mode == abi.BILLBOARD_UP_CAMERA_Y else np.array([0, 1, 0], F32)
    base = billboard_base(M, cam_pos, up, locks)
    if abs(np.linalg.det(base[:3, :3].astype(np.float64))) < 1e-6:
        # a lock against a LookAt straight up flattens the matrix; the plain model
        # under it has no inverse for its depth keys, so the equivalence does not
        # apply (the GPU test compares that case with the oracle directly)
        assert cam_kind == "down" and any(locks)
        return
    got = pyoracle.render(_scene(mat, M), cam)
    plain = scenes.default_material(shadeless=1, backface_culling=0)
    ref = pyoracle.render(_scene(plain, base), cam)
    assert ref.visible_tris > 0
    gt, gx, gd = _by_tri(got)
    rt, rx, rd = _by_tri(ref)
    assert np.array_equal(gt, rt) and np.array_equal(gx, rx) and np.array_equal(gd, rd)
    # DepthModeUnbillboarded: same corners, the depth of the unturned model
    mat["billboard_depth"] = abi.DEPTH_UNBILLBOARDED
    ub = pyoracle.render(_scene(mat, M), cam)
    _, ux, ud = _by_tri(ub)
    assert np.array_equal(ux, gx)
    # the unturned part's per-vertex depth, from the same corners' vertices
    raw = pyoracle.render(_scene(plain, M), cam)
    q = scenes.quad_mesh(1.5, 1.0)
    vdepth = {}
    for t, dep in zip(raw.tri_index, raw.depth):
        for k in range(3):
            vdepth[int(q.indices[t, k])] = dep[k]
    for t, dep in zip(ub.tri_index, ub.depth):
        for k in range(3):
            v = int(q.indices[t, k])
            if v in vdepth:
                assert dep[k] == vdepth[v]


def test_billboard_faces_the_camera():
    """Unlocked, a quad under an identity model rotation turns its +Z face to the camera."""
    cam = scenes.feature_camera("tilted")
    cam_pos = np.asarray(cam.transform[:], F32).reshape(4, 4)[3, :3]
    for p in ([4.0, 1.0, -10.0], [-6.0, -2.0, -20.0]):
        M = scenes.trs(np.array(p, F32), np.ones(3, F32), scenes.ident())[0]
        base = billboard_base(M, cam_pos, np.array([0, 1, 0], F32), (0, 0, 0))
        n = base[2, :3].astype(np.float64)
        d = (cam_pos - np.array(p)).astype(np.float64)
        assert np.dot(n, d) / np.linalg.norm(d) > 0.999
