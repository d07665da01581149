"""Dynamic batching in the oracle (Model.DynamicBatchAdd; Camera.Render's pair
collection camera.go:1343-1457 and batch drawing camera.go:2068-2093):
members draw only inside their owner's batch, far to near from the camera, all
of their parts, as one flush; owners draw no mesh of their own; a batch whose
owner is itself batched is never drawn; each member part renders exactly as it
would unbatched."""
import numpy as np

from oracle import pyoracle
from tetra3d_gb300 import scenes


def _frame(sd, variant="persp"):
    return pyoracle.render(sd, scenes.feature_camera(variant))


def test_batch_structure():
    sd = scenes.batch_scene(11)
    n = sd.nmodels
    r = _frame(sd)
    models = [s["model"] for s in r.segments]
    assert 0 not in models and 1 not in models  # owners
    assert 2 in models  # a nested owner drawn as a member
    assert n - 12 not in models  # the member of the nested owner
    assert 5 not in models and 9 not in models  # invisible members
    assert not any(s["count"] for s in r.segments if s["model"] == 7)  # culled inside its batch
    draws = {}
    for s in r.segments:
        draws.setdefault(s["draw"], []).append(s)
    batched = [v for v in draws.values() if v[0]["model"] >= 2 and sd.mv["batched"][v[0]["model"]]]
    assert len(batched) == 4
    cam = scenes.feature_camera("persp")
    cp = np.asarray(cam.transform[:], np.float32).reshape(4, 4)[3, :3]
    for v in batched:
        seen, dist = [], []
        for s in v:
            if s["model"] not in seen:
                seen.append(s["model"])
                p = sd.mv["transform"][s["model"]].reshape(4, 4)[3, :3]
                dist.append(float(np.sum((cp - p).astype(np.float32) ** 2)))
            # every part of a member, in part order
        assert all(a >= b for a, b in zip(dist, dist[1:]))  # far to near
        owners = {int(sd.mv["batch_owner"][m]) for m in seen}
        assert len(owners) == 1
        for m in seen:
            nparts = len(sd.meshes[int(sd.mv["mesh"][m])].parts)
            assert [s["part"] for s in v if s["model"] == m] == list(range(nparts))
        assert len({s["draw_transparent"] for s in v}) == 1


def test_member_parts_render_as_unbatched():
    sd = scenes.batch_scene(11)
    r = _frame(sd, "tilted")
    plain = scenes.batch_scene(11)
    plain.mv["batched"] = 0
    q = _frame(plain, "tilted")

    def by_pair(f):
        out, b = {}, 0
        for s in f.segments:
            out[(s["model"], s["part"])] = (f.xyuv[b:b + s["count"]], f.rgba[b:b + s["count"]], f.depth[b:b + s["count"]])
            b += s["count"]
        return out

    a, b = by_pair(r), by_pair(q)
    compared = 0
    for key, va in a.items():
        if key in b:  # parts with an invisible material draw only inside a batch
            for x, y in zip(va, b[key]):
                assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), key
            compared += 1
    assert compared > 20


def test_batches_without_members_draw_normally():
    sd = scenes.batch_scene(11)
    sd.mv["batched"] = 0
    r = _frame(sd)
    assert 0 in {s["model"] for s in r.segments}
    assert len({s["draw"] for s in r.segments}) == len(r.segments)
