"""The rasteriser's oracle (oracle/t3d_oracle_raster.cpp) on hand-built frames with known
answers: the fill rule covers a split quad exactly once, the depth encoding round trip, the
per-pair depth test, transparent pairs that do not write depth, and the plain draw with depth
rendering off. No GPU needed."""
import types

import numpy as np

from tetra3d_gb300 import scenes
from oracle import pyoracle

F = np.float32


def _frame(tris):
    """tris: list of (pair, [(x, y)] * 3, (r, g, b, a), depth) -> a frame in draw order."""
    n = len(tris)
    xyuv = np.zeros((n, 3, 4), F)
    rgba = np.zeros((n, 3, 4), F)
    depth = np.zeros((n, 3), F)
    segs = []
    for i, (pair, pts, col, d) in enumerate(tris):
        xyuv[i, :, 0:2] = pts
        rgba[i, :, :] = col
        depth[i, :] = d
        if not segs or segs[-1]["pair"] != pair:
            segs.append(dict(pair=pair, count=0))
        segs[-1]["count"] += 1
    return types.SimpleNamespace(xyuv=xyuv, rgba=rgba, depth=depth, segments=segs)


def _cam(w=16, h=16, render_depth=1, fog_on=0):
    return scenes.camera(w=w, h=h, render_depth=render_depth, fog_on=fog_on)


def _q8(v):
    return int(np.floor(np.clip(F(v), 0, 1) * F(255) + F(0.5)))


def test_split_quad_is_covered_once():
    quad = [(2, 2), (10, 2), (10, 10), (2, 10)]
    col = (1.0, 1.0, 1.0, 0.5)  # half alpha: a double-covered pixel would blend twice
    f = _frame([(0, [quad[0], quad[1], quad[2]], col, 0.5), (0, [quad[0], quad[2], quad[3]], col, 0.5)])
    for rd in (1, 0):
        c, d = pyoracle.raster(f, None, _cam(render_depth=rd), transparent=[0])
        cov = c[..., 3] > 0
        assert cov.sum() == 64, rd
        assert np.all(c[cov] == [_q8(0.5), _q8(0.5), _q8(0.5), _q8(0.5)])
        assert cov[2:10, 2:10].all()


def test_depth_encoding_round_trip():
    f = _frame([(0, [(0, 0), (16, 0), (0, 16)], (1, 0, 0, 1), 0.5)])
    c, d = pyoracle.raster(f, None, _cam(), transparent=[0])
    px = d[1, 1]
    assert list(px) == [127, 127, 128, 255]  # encodeDepth(0.5) written as unorm8
    dec = F(px[0]) / F(255) + (F(px[1]) / F(255)) / F(255) + (F(px[2]) / F(255)) / F(65025)
    assert abs(float(dec) - 0.5) < 1e-5
    assert list(c[1, 1]) == [255, 0, 0, 255]


def test_depth_test_between_pairs():
    tri = [(0, 0), (16, 0), (0, 16)]
    near, far = ((0, 1, 0, 1), 0.2), ((1, 0, 0, 1), 0.8)
    f = _frame([(0, tri, *far), (1, tri, *near)])   # far first: near overwrites
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0, 0])
    assert list(c[1, 1]) == [0, 255, 0, 255]
    f = _frame([(0, tri, *near), (1, tri, *far)])   # near first: far fails the test
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0, 0])
    assert list(c[1, 1]) == [0, 255, 0, 255]
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[1, 0])  # a transparent near pair writes no depth
    assert list(c[1, 1]) == [255, 0, 0, 255]


def test_plain_draw_without_depth_is_painter_order():
    tri = [(0, 0), (16, 0), (0, 16)]
    f = _frame([(0, tri, (0, 1, 0, 1), 0.2), (1, tri, (1, 0, 0, 1), 0.8)])
    c, d = pyoracle.raster(f, None, _cam(render_depth=0), transparent=[0, 0])
    assert list(c[1, 1]) == [255, 0, 0, 255]
    assert d.max() == 0


def test_fog_add_by_depth():
    cam = _cam(fog_on=1)
    cam.fog_range[:] = [0.0, 1.0]
    cam.fog_color[:] = [0.0, 0.0, 1.0, 1.0]
    f = _frame([(0, [(0, 0), (16, 0), (0, 16)], (1, 0, 0, 1), 1.0)])
    c, _ = pyoracle.raster(f, None, cam, transparent=[0])
    assert list(c[1, 1]) == [255, 0, 255, 255]  # smoothstep(0, 1, ~1) = 1: full fog colour added
