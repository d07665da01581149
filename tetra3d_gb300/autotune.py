"""Autotuner for the batched frame.

Sweeps the launch shape of a frame -- one launch per phase or the whole frame in
one cooperative persistent launch (t3d_set_split_phases) -- against triangles per
tile (the unit of the visibility / sort / emit work queues; for meshlet frames
also the meshlet size, so each tile size re-cuts the scene's meshlets) and threads
per block, on the caller's own scene and camera, timing captured-graph replays
with CUDA events, then the vertices per vertex-phase work item of the per-vertex
record route, and leaves the context on the fastest setting. The 512-bin sort
itself is fixed by the reference's bucket sort (sortingTriangles.go:166-168), so
its radix is not a free parameter.
"""
import ctypes as C
import itertools
import time

TILES = (1024, 2048)
BLOCKS = (256,)
SPLITS = (1, 0)
CHUNKS = (2048, 4096, 8192)


def time_config(ctx, sid, cam, tile, block, frames=10, warmup=3, animate=False, split=None):
    import torch
    ctx.set_tuning(tile_tris=tile, block_threads=block)
    if split is not None:
        ctx.set_split_phases(split)
    ctx.graph_capture(sid, cam, animate=animate)
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    ctx.graph_replay(warmup, stream=sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.graph_replay(frames, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / frames


def tune(ctx, sid, cam, frames=10, tiles=TILES, blocks=BLOCKS, splits=SPLITS, chunks=CHUNKS, animate=False,
         verbose=False):
    """Returns (best (tile, block, split, vertex chunk), {config: ms per frame}); leaves ctx tuned
    to the best. chunks=() skips the vertex-chunk stage (frames whose pairs all take meshlets)."""
    results = {}
    t0 = time.time()
    for tile, block, split in itertools.product(tiles, blocks, splits):
        try:
            ms = time_config(ctx, sid, cam, tile, block, frames=frames, animate=animate, split=split)
        except Exception as exc:  # a shape that does not fit (occupancy) is skipped
            if verbose:
                print(f"autotune: tile {tile} block {block} split {split} skipped: {exc}")
            continue
        results[(tile, block, split)] = ms
        if verbose:
            print(f"autotune: tile {tile:5d} block {block:3d} split {split}: {ms:.3f} ms/frame")
    best = min(results, key=results.get)
    ctx.set_tuning(tile_tris=best[0], block_threads=best[1])
    ctx.set_split_phases(best[2])
    bch = 0
    if chunks:
        # second stage: the vertex chunk at the best shape
        chunk_ms = {}
        for ch in chunks:
            ctx.set_tuning(vertex_chunk=ch)
            chunk_ms[ch] = time_config(ctx, sid, cam, best[0], best[1], frames=frames, animate=animate)
            results[best + (ch,)] = chunk_ms[ch]
            if verbose:
                print(f"autotune: {best} chunk {ch:5d}: {chunk_ms[ch]:.3f} ms/frame")
        bch = min(chunk_ms, key=chunk_ms.get)
        ctx.set_tuning(vertex_chunk=bch)
    best = best + (bch,)
    if verbose:
        print(f"autotune: best {best} in {time.time() - t0:.1f} s")
    return best, results
