"""TEST INFRASTRUCTURE ONLY: binary32 error of the vertex stage against the oracle's
binary64 twin, on the benchmark configurations.

The GPU library matches the binary32 oracle bit for bit (tests/), so the binary32
oracle's error against the binary64 twin (t3d_oracle_render_f64: every operation of
the same restatement in double precision) is the GPU's error. Per configuration:

- boundary triangles: kept by one precision and dropped by the other (near/far,
  +-0.5, backface or NaN tests within rounding of their threshold), counted against
  the binary32 visible total;
- for triangles both keep: the largest error of each emitted attribute, in units of
  the binary32 spacing at the binary64 value (ulp) where |value| >= a floor, and as
  an absolute error;
- sort order: render pairs whose common triangles come out in a different order
  (a depth key within rounding of a bin edge moves a triangle to the next bin).

python -m oracle.f64_report [config ...]   (configs: sphere cubes terrain batched)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from oracle import pyoracle  # noqa: E402
from tetra3d_gb300 import scenes  # noqa: E402

FLOORS = {"screen xy": 64.0, "uv": 1e-3, "rgba": 1e-3, "depth": 1e-3}  # ulp where |value| >= floor


def _attrs(f, rows):
    x = f.xyuv[rows]
    return {"screen xy": x[..., :2], "uv": x[..., 2:], "rgba": f.rgba[rows], "depth": f.depth[rows]}


def compare(sd, cam, threads, animate_frames=0):
    a = pyoracle.render(sd, cam, threads=threads, animate_frames=animate_frames)
    b = pyoracle.render(sd, cam, threads=threads, animate_frames=animate_frames, f64=True)
    boundary = 0
    reordered = 0
    ra, rb = [], []
    ia = ib = 0
    for sa, sb in zip(a.segments, b.segments):
        assert (sa["model"], sa["part"]) == (sb["model"], sb["part"])
        ta = a.tri_index[ia:ia + sa["count"]]
        tb = b.tri_index[ib:ib + sb["count"]]
        common = np.intersect1d(ta, tb, assume_unique=True)
        boundary += len(ta) + len(tb) - 2 * len(common)
        if len(common) == len(ta) == len(tb):  # the common case: same set
            if not np.array_equal(ta, tb):
                reordered += 1
            pos_b = np.empty(0, np.int64)
            order = np.argsort(tb, kind="stable")
            pos_b = ib + order[np.searchsorted(tb[order], ta)]
            ra.append(np.arange(ia, ia + len(ta)))
            rb.append(pos_b)
        else:
            ka = np.isin(ta, common)
            kb = np.isin(tb, common)
            if not np.array_equal(ta[ka], tb[kb]):
                reordered += 1
            sel_a = np.nonzero(ka)[0]
            order = np.argsort(tb, kind="stable")
            ra.append(ia + sel_a)
            rb.append(ib + order[np.searchsorted(tb[order], ta[sel_a])])
        ia += sa["count"]
        ib += sb["count"]
    ra = np.concatenate(ra) if ra else np.zeros(0, np.int64)
    rb = np.concatenate(rb) if rb else np.zeros(0, np.int64)
    A, B = _attrs(a, ra), _attrs(b, rb)
    out = {"visible_f32": a.visible_tris, "boundary": boundary, "pairs": len(a.segments), "reordered_pairs": reordered}
    for k in A:
        x = A[k].astype(np.float64)
        y = B[k]
        err = np.abs(x - y)
        big = np.abs(y) >= FLOORS[k]
        sp = np.spacing(np.abs(y[big]).astype(np.float32)).astype(np.float64)
        out[k] = {"max_abs": float(err.max()) if err.size else 0.0,
                  "max_ulp": float((err[big] / sp).max()) if big.any() else 0.0,
                  "p99_ulp": float(np.percentile(err[big] / sp, 99)) if big.any() else 0.0}
    return out


CONFIGS = {
    "sphere": lambda: scenes.uv_sphere_scene(1),
    "cubes": lambda: scenes.cubes_scene(2),
    "terrain": lambda: scenes.terrain_scene(3),
    "batched": lambda: scenes.batched_scene(4),
}


def main(names):
    threads = os.cpu_count() or 1
    print("| config | visible (binary32) | boundary triangles | pairs reordered | max ulp (p99): screen xy / uv / rgba / depth | max abs: screen xy (px) / depth |")
    print("|---|---|---|---|---|---|")
    for name in names:
        t0 = time.time()
        sd = CONFIGS[name]()
        r = compare(sd, sd.camera, threads)
        ulps = " / ".join(f"{r[k]['max_ulp']:.1f} ({r[k]['p99_ulp']:.1f})" for k in ("screen xy", "uv", "rgba", "depth"))
        print(f"| {name} | {r['visible_f32']} | {r['boundary']} ({r['boundary'] / max(1, r['visible_f32']):.2e}) | "
              f"{r['reordered_pairs']} of {r['pairs']} | {ulps} | {r['screen xy']['max_abs']:.3g} / {r['depth']['max_abs']:.3g} |",
              flush=True)
        print(f"<!-- {name}: {time.time() - t0:.0f} s -->", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CONFIGS))
