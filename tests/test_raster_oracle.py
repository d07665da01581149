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


# ---- textures and alpha clip (base3d.kage, the clip-alpha shader of camera.go:390-480) ----

def _tex(w=4, h=4, alpha=None, seed=0):
    """A premultiplied RGBA8 texture with distinct texels."""
    rng = np.random.default_rng(seed)
    a = np.full((h, w), 255, np.uint8) if alpha is None else np.asarray(alpha, np.uint8)
    rgb = (rng.integers(0, 256, (h, w, 3)) * (a[..., None] / 255.0)).astype(np.uint8)
    return np.ascontiguousarray(np.concatenate([rgb, a[..., None]], -1))


def _quad(x0, y0, x1, y1, u0, v0, u1, v1, col=(1, 1, 1, 1), d=0.5, pair=0):
    """Two triangles of a screen rectangle with SrcX/SrcY spread linearly over it."""
    pts = [(x0, y0, u0, v0), (x1, y0, u1, v0), (x1, y1, u1, v1), (x0, y1, u0, v1)]
    return [(pair, [pts[0], pts[1], pts[2]], col, d), (pair, [pts[0], pts[2], pts[3]], col, d)]


def _uv_frame(tris):
    n = len(tris)
    xyuv = np.zeros((n, 3, 4), F)
    rgba = np.zeros((n, 3, 4), F)
    depth = np.zeros((n, 3), F)
    segs = []
    for i, (pair, pts, col, d) in enumerate(tris):
        xyuv[i] = pts
        rgba[i] = col
        depth[i] = d
        if not segs or segs[-1]["pair"] != pair:
            segs.append(dict(pair=pair, count=0))
        segs[-1]["count"] += 1
    return types.SimpleNamespace(xyuv=xyuv, rgba=rgba, depth=depth, segments=segs)


def test_nearest_texture_maps_texels_to_pixels():
    t = _tex()
    f = _uv_frame(_quad(2, 2, 6, 6, 0, 0, 4, 4))
    for rd in (1, 0):
        c, _ = pyoracle.raster(f, None, _cam(render_depth=rd), transparent=[0], textures=[t], flush_tex=[(1, 0, (1, 1))])
        assert np.array_equal(c[2:6, 2:6], t), rd


def test_texture_wraps_and_multiplies_the_vertex_colour():
    t = _tex(seed=1)
    f = _uv_frame(_quad(0, 0, 8, 8, -4, 0, 4, 8, col=(0.5, 1.0, 1.0, 1.0)))  # u from -4: mod wraps
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 0, (1, 1))])
    want = np.tile(t, (2, 2, 1))
    assert np.array_equal(c[0:8, 0:8, 1:], want[..., 1:])
    assert np.array_equal(c[0:8, 0:8, 0], np.floor(want[..., 0] / 255.0 * 0.5 * 255 + 0.5).astype(np.uint8))


def test_bilinear_at_texel_centres_is_nearest_and_halfway_is_the_mean():
    t = _tex(seed=2)
    f = _uv_frame(_quad(0, 0, 4, 4, 0, 0, 4, 4))
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 1, (1, 1))])
    assert np.array_equal(c[0:4, 0:4], t)
    f = _uv_frame(_quad(0, 0, 4, 4, 0.5, 0, 4.5, 4))  # sample points on the texel edges in x
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 1, (1, 1))])
    mean = (t[:, :, :].astype(np.float64) + np.roll(t, -1, axis=1)) / 2.0
    assert np.abs(c[0:4, 0:4].astype(np.float64) - mean).max() <= 1.0


def test_screen_mapped_texture_ignores_the_uv():
    t = _tex(seed=3)
    f = _uv_frame(_quad(0, 0, 8, 8, 0, 0, 0, 0))
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 2, (1, 1))])
    assert np.array_equal(c[0:8, 0:8], np.tile(t, (2, 2, 1)))


def test_alpha_clip_drops_low_alpha_texels_from_depth_and_colour():
    alpha = np.full((4, 4), 255, np.uint8)
    alpha[0, :] = 204   # 0.8: dropped (tex.a <= 0.8)
    alpha[1, :] = 230   # 0.902: kept, blended into the intermediate at that alpha
    t = _tex(alpha=alpha, seed=4)
    f = _uv_frame(_quad(0, 0, 4, 4, 0, 0, 4, 4))
    c, d = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 4, (1, 1))])
    assert d[0, 0:4, 3].max() == 0 and c[0, 0:4].max() == 0
    assert np.all(d[1, 0:4, 3] == 230) and np.all(d[2:4, 0:4, 3] == 255)
    assert np.array_equal(c[1:4, 0:4], t[1:4])
    # without the clip every texel draws and writes depth
    c, d = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 0, (1, 1))])
    assert np.all(d[0:4, 0:4, 3] == 255) and np.array_equal(c[0:4, 0:4], t)


def test_alpha_clip_lets_a_far_pair_show_through_the_holes():
    alpha = np.full((4, 4), 255, np.uint8)
    alpha[:, 0] = 0
    t = _tex(alpha=alpha, seed=5)
    near = _quad(0, 0, 4, 4, 0, 0, 4, 4, d=0.2, pair=0)
    far = _quad(0, 0, 4, 4, 0, 0, 4, 4, col=(0, 1, 0, 1), d=0.8, pair=1)
    f = _uv_frame(near + far)
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0, 0], textures=[t],
                           flush_tex=[(1, 4, (1, 1)), (0, 0, (1, 1))])
    assert np.all(c[0:4, 0] == [0, 255, 0, 255])  # the hole: the far pair passes the depth test
    assert np.array_equal(c[0:4, 1:4], t[:, 1:4])


def test_bilinear_wraps_across_the_texture_edge():
    """A sample point on the seam between the last and the first column mixes the two (GLSL mod
    wrapping of both taps, rate = fract(p1)); nearest takes the texel containing the point."""
    t = _tex(w=4, h=1, seed=6)
    # a one-pixel-high strip: pixel centres at x + 0.5 map to u = x + 0.5 + 3.5, i.e. on the seams
    f = _uv_frame(_quad(0, 0, 4, 1, 3.5, 0.5, 7.5, 0.5))
    c, _ = pyoracle.raster(f, None, _cam(w=4, h=1), transparent=[0], textures=[t], flush_tex=[(1, 1, (1, 1))])
    row = t[0].astype(np.float64)
    for x in range(4):
        want = (row[(x + 3) % 4] + row[x % 4]) / 2.0
        assert np.abs(c[0, x].astype(np.float64) - want).max() <= 1.0, x
    c, _ = pyoracle.raster(f, None, _cam(w=4, h=1), transparent=[0], textures=[t], flush_tex=[(1, 0, (1, 1))])
    assert np.array_equal(c[0], t[0, [0, 1, 2, 3]])


def test_negative_coordinates_wrap_with_mod():
    """u = -0.5 lands in the last texel (mod, not remainder)."""
    t = _tex(w=4, h=4, seed=7)
    f = _uv_frame(_quad(0, 0, 4, 4, -4, -4, 0, 0))
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 0, (1, 1))])
    assert np.array_equal(c[0:4, 0:4], t)


def test_screen_mapping_scales_the_pixel_position():
    """TextureMapMode 1 with multipliers (0.5, 0.5): two pixels per texel in each direction."""
    t = _tex(w=4, h=4, seed=8)
    f = _uv_frame(_quad(0, 0, 8, 8, 0, 0, 0, 0))
    c, _ = pyoracle.raster(f, None, _cam(), transparent=[0], textures=[t], flush_tex=[(1, 2, (0.5, 0.5))])
    assert np.array_equal(c[0:8, 0:8], np.repeat(np.repeat(t, 2, axis=0), 2, axis=1))


def test_alpha_clip_on_a_transparent_flush_writes_no_depth():
    """A transparent flush with alpha clip: the clipped texels still gate its colour pass, but
    its depth intermediate is not composited into the depth texture."""
    alpha = np.full((4, 4), 255, np.uint8)
    alpha[:, :2] = 0
    t = _tex(alpha=alpha, seed=9)
    f = _uv_frame(_quad(0, 0, 4, 4, 0, 0, 4, 4))
    c, d = pyoracle.raster(f, None, _cam(), transparent=[1], textures=[t], flush_tex=[(1, 4, (1, 1))])
    assert d.max() == 0
    assert c[0:4, 0:2].max() == 0 and np.array_equal(c[0:4, 2:4], t[:, 2:4])
