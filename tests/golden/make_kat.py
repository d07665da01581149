"""Generates tests/golden/kat_single_triangles.json: known answers for one-triangle scenes.

The expected values are computed here with plain numpy binary32 scalar
arithmetic written directly from the reference formulas (camera.go:638-679,
:1646-1820; model.go:600-995; light.go:110-360; matrix.go:588-637), independently
of the C++ oracle, so the oracle can be pinned against them. Run from the repo
root: python tests/golden/make_kat.py
"""
import json
import math
import os

import numpy as np

F = np.float32
HERE = os.path.dirname(os.path.abspath(__file__))


def f(x):
    return F(x)


def mm(a, b):  # Matrix4.Mult (matrix_none.go:6-32)
    o = np.zeros((4, 4), F)
    for i in range(4):
        for j in range(4):
            o[i, j] = ((a[i, 0] * b[0, j] + a[i, 1] * b[1, j]) + a[i, 2] * b[2, j]) + a[i, 3] * b[3, j]
    return o


def mvw(m, v):  # MultVecW (matrix.go:630-636)
    x, y, z = v
    return [((m[0, c] * x + m[1, c] * y) + m[2, c] * z) + m[3, c] for c in range(4)]


def camera_vp(W, H, fov, near, far):
    """Camera at the origin with identity rotation: View = T(-0) * I^T, times the perspective matrix."""
    aspect = f(W) / f(H)
    t = f(math.tan(float(f(fov) * f(math.pi) / f(360))))
    r = t * aspect
    P = np.zeros((4, 4), F)
    P[0, 0] = (f(2) * f(near)) / (r - (-r))
    P[0, 2] = (r + (-r)) / (r - (-r))
    P[1, 1] = (f(2) * f(near)) / (t - (-t))
    P[1, 2] = (t + (-t)) / (t - (-t))
    P[2, 2] = -((f(far) + f(near)) / (f(far) - f(near)))
    P[2, 3] = -((f(2) * f(far) * f(near)) / (f(far) - f(near)))
    P[3, 2] = f(-1)
    V = np.eye(4, dtype=F)
    V[3, :3] = [-0.0, -0.0, -0.0]
    return mm(mm(V, np.eye(4, dtype=F).T.copy()), P)


def unit(v):  # Vector3.Unit
    l = F(math.sqrt(float(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])))
    if l < F(1e-8) or l == F(1):
        return v
    return [v[0] / l, v[1] / l, v[2] / l]


def case(name, tri, uv=None, light=None, expect_visible=True):
    W, H, fov, near, far = 640, 360, 60.0, 0.1, 100.0
    vp = camera_vp(W, H, fov, near, far)  # model transform is identity: mvp = I * vp
    M = np.eye(4, dtype=F)
    mvp = mm(M, vp)
    clip = [mvw(mvp, [f(c) for c in p]) for p in tri]
    vis = False
    for c in clip:
        if c[2] + F(1) >= F(near) and c[2] < F(far):
            vis = True
    tv = []
    for c in clip:
        w = c[3] if c[3] >= 0 else F(0.000001)
        tv.append((c[0] / w, c[1] / w))
    if vis:
        for ax in (0, 1):
            if all(p[ax] < F(-0.5) for p in tv) or all(p[ax] > F(0.5) for p in tv):
                vis = False
    if vis:
        n0x, n0y = tv[0][0] - tv[1][0], tv[0][1] - tv[1][1]
        n1x, n1y = tv[1][0] - tv[2][0], tv[1][1] - tv[2][1]
        if (n0x * n1y) - (n1x * n0y) < F(0):
            vis = False
    assert vis == expect_visible, name
    # without a light the material is shadeless, so the colour stays the unlit model colour
    out = {"name": name, "positions": [[float(x) for x in p] for p in tri], "visible": vis, "light": light,
           "shadeless": light is None}
    if not vis:
        return out
    margin = (F(far) - F(near)) * F(0.04)
    spread = F(far) - F(near) + (margin * F(2))
    uv = uv or [[0.25, 0.75], [0.5, 0.5], [1.0, 0.0]]
    corners = []
    normal = [F(0), F(0), F(1)]
    for vi, c in enumerate(clip):
        w = c[3] if c[3] >= 0 else F(0.001)
        dx = (c[0] / w) * F(W) + F(W) / F(2)
        dy = (c[1] / -w) * F(H) + F(H) / F(2)
        u, v = F(uv[vi][0]), F(uv[vi][1])
        su, sv = u * F(64), (F(1) - v) * F(32)
        depth = (c[2] + margin) / spread
        depth = F(0) if depth < 0 else (F(1) if depth > 1 else depth)
        r = g = b = F(1)
        a = F(1)
        if light is not None:
            lr = lg = lb = F(0)
            p = [F(x) for x in tri[vi]]
            if light["type"] == "ambient":
                e = F(light["energy"])
                lr, lg, lb = F(0) + F(1) * e, F(0) + F(1) * e, F(0) + F(1) * e
            elif light["type"] == "point":
                wp = [F(x) for x in light["pos"]]
                dd = [wp[0] - p[0], wp[1] - p[1], wp[2] - p[2]]
                dist = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]
                R2 = F(light["range"]) * F(light["range"])
                if not dist > R2:
                    lv = unit(dd)
                    diffuse = normal[0] * lv[0] + normal[1] * lv[1] + normal[2] * lv[2]
                    if diffuse > 0:
                        df = diffuse * (F(1) / (F(1) + (F(0.1) * dist))) * F(2)
                        dc = (R2 - dist) / dist
                        dc = F(0) if dc < 0 else (F(1) if dc > 1 else dc)
                        df = df * dc
                        E = F(light["energy"])
                        lr = F(0) + F(1) * df * E
                        lg, lb = lr, lr
            r, g, b = r * lr, g * lg, b * lb
        corners.append([float(x) for x in (dx, dy, su, sv, r, g, b, a, depth)])
    out["corners"] = corners
    return out


def main():
    front = [[-1.0, -1.0, -5.0], [1.0, -1.0, -5.0], [0.0, 1.0, -5.0]]
    cases = [
        case("front_facing_unlit", front),
        case("back_facing", [front[0], front[2], front[1]], expect_visible=False),
        case("behind_camera", [[-1.0, -1.0, 5.0], [1.0, -1.0, 5.0], [0.0, 1.0, 5.0]], expect_visible=False),
        case("off_screen_right", [[40.0, -1.0, -5.0], [42.0, -1.0, -5.0], [41.0, 1.0, -5.0]], expect_visible=False),
        case("beyond_far_plane", [[-1.0, -1.0, -150.0], [1.0, -1.0, -150.0], [0.0, 1.0, -150.0]],
             expect_visible=False),
        case("ambient_lit", front, light={"type": "ambient", "energy": 0.25}),
        case("point_lit", front, light={"type": "point", "pos": [0.5, 0.0, -2.0], "range": 10.0, "energy": 2.0}),
    ]
    with open(os.path.join(HERE, "kat_single_triangles.json"), "w") as fh:
        json.dump({"camera": {"w": 640, "h": 360, "fov": 60.0, "near": 0.1, "far": 100.0},
                   "texture": [64, 32], "cases": cases}, fh, indent=1)


if __name__ == "__main__":
    main()
