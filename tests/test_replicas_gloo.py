"""The N>1 host path on CPU: two gloo ranks, each rendering its share of the models
(oracle), combine timing and totals as bench.py does under torchrun; the combined
totals and the per-pair results equal one rank rendering everything."""
import json
import os
import socket

import numpy as np
import pytest

from tetra3d_gb300 import replicas, scenes

WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    from oracle import pyoracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sd = scenes.feature_scene(9)
    cam = scenes.feature_camera("tilted")
    mine = replicas.shard_models(sd.nmodels, rank, world)
    f = pyoracle.render(scenes.subset(sd, mine), cam)
    fake_ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    ms, units, nbytes = replicas.combine(fake_ms, f.visible_tris, 100 * (rank + 1), dist)
    pairs, b = {}, 0
    for s in f.segments:
        key = f"{int(mine[s['model']])}/{s['part']}"
        pairs[key] = f.xyuv[b:b + s["count"]].view(np.uint32).sum(dtype=np.uint64).item()
        b += s["count"]
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fh:
        json.dump({"ms": ms, "units": units, "bytes": nbytes, "pairs": pairs}, fh)
    dist.barrier()
    dist.destroy_process_group()


def test_shard_models_partitions():
    for n in (0, 1, 7, 4096):
        for w in (1, 2, 3, 8):
            got = np.concatenate([replicas.shard_models(n, r, w) for r in range(w)])
            assert np.array_equal(got, np.arange(n))
    with pytest.raises(ValueError):
        replicas.shard_models(4, 2, 2)


def test_two_gloo_ranks_combine_like_one(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    from oracle import pyoracle
    mp.start_processes(_rank_main, args=(WORLD, _free_port(), str(tmp_path)), nprocs=WORLD, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(WORLD)]
    sd = scenes.feature_scene(9)
    cam = scenes.feature_camera("tilted")
    whole = pyoracle.render(sd, cam)
    for r in res:
        assert r["ms"] == 15.0, "max over ranks"
        assert r["units"] == whole.visible_tris, "sum over ranks"
        assert r["bytes"] == 300
    b, want = 0, {}
    for s in whole.segments:
        want[f"{s['model']}/{s['part']}"] = whole.xyuv[b:b + s["count"]].view(np.uint32).sum(dtype=np.uint64).item()
        b += s["count"]
    got = {}
    for r in res:
        got.update(r["pairs"])
    assert got == want
