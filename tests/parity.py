"""Comparison helpers for GPU frames against the oracle."""
import numpy as np


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_frames_equal(got, ref, what=""):
    """Bit-exact comparison: draw order, per-segment counts and every emitted float."""
    gs = [(s["model"], s["part"], s["count"]) for s in got.segments]
    rs = [(s["model"], s["part"], s["count"]) for s in ref.segments]
    assert len(gs) == len(rs), f"{what}: {len(gs)} segments vs oracle {len(rs)}"
    bad = [(i, g, r) for i, (g, r) in enumerate(zip(gs, rs)) if g != r]
    assert not bad, f"{what}: segment mismatch (index, gpu, oracle) {bad[:5]}"
    assert got.visible_tris == ref.visible_tris, f"{what}: visible {got.visible_tris} vs {ref.visible_tris}"
    for name in ("xyuv", "rgba", "depth"):
        a, b = bits(getattr(got, name)), bits(getattr(ref, name))
        if not np.array_equal(a, b):
            diff = np.argwhere(a.reshape(a.shape[0], -1) != b.reshape(b.shape[0], -1))
            t = int(diff[0, 0])
            raise AssertionError(f"{what}: {name} differs at {len(diff)} places; first triangle {t}: "
                                 f"gpu {getattr(got, name)[t]} oracle {getattr(ref, name)[t]}")


def max_rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.maximum(np.abs(b), 1e-6)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0
