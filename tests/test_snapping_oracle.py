"""Camera.VertexSnapping in the oracle (model.go:813-818): clip X, Y and Z are
rounded to multiples of 1/VertexSnapping before the divide, so with an
orthographic camera (w = 1) every emitted screen position sits on that grid,
and snapping off or at a fine enough grid changes nothing visible."""
import numpy as np

from oracle import pyoracle
from tetra3d_gb300 import scenes


def test_orthographic_positions_on_the_grid():
    sd = scenes.feature_scene(5)
    cam = scenes.feature_camera("ortho")
    cam.vertex_snapping = 4.0
    r = pyoracle.render(sd, cam)
    assert r.visible_tris > 0
    W, H = float(cam.width), float(cam.height)
    gx = (r.xyuv[:, :, 0].astype(np.float64) - W / 2) / W * 4.0
    gy = -(r.xyuv[:, :, 1].astype(np.float64) - H / 2) / H * 4.0
    assert np.abs(gx - np.round(gx)).max() < 1e-3
    assert np.abs(gy - np.round(gy)).max() < 1e-3
    plain = pyoracle.render(sd, scenes.feature_camera("ortho"))
    assert not np.array_equal(plain.xyuv, r.xyuv)


def test_snapping_off_is_the_default():
    sd = scenes.feature_scene(6)
    a = pyoracle.render(sd, scenes.feature_camera("persp"))
    cam = scenes.feature_camera("persp")
    cam.vertex_snapping = 0.0
    b = pyoracle.render(sd, cam)
    assert np.array_equal(a.xyuv.view(np.uint32), b.xyuv.view(np.uint32))
    cam.vertex_snapping = -1.0  # VertexSnapping <= 0 is off
    c = pyoracle.render(sd, cam)
    assert np.array_equal(a.xyuv.view(np.uint32), c.xyuv.view(np.uint32))
