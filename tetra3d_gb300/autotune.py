"""Autotuner for the batched frame kernel.

Sweeps the launch shape knobs of the persistent kernel -- triangles per tile
(the unit of the visibility / sort / emit work queues) and threads per block,
then vertices per vertex-phase work item -- on the caller's own scene and
camera, timing captured-graph replays with CUDA events, and leaves the context
on the fastest setting. The 512-bin sort itself
is fixed by the reference's bucket sort (sortingTriangles.go:166-168), so its
radix is not a free parameter.
"""
import ctypes as C
import itertools
import time

TILES = (1024, 2048, 4096)
BLOCKS = (128, 256)
CHUNKS = (2048, 4096, 8192)


def time_config(ctx, sid, cam, tile, block, frames=10, warmup=3, animate=False):
    import torch
    ctx.set_tuning(tile_tris=tile, block_threads=block)
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


def tune(ctx, sid, cam, frames=10, tiles=TILES, blocks=BLOCKS, chunks=CHUNKS, animate=False, verbose=False):
    """Returns (best (tile, block, vertex chunk), {config: ms per frame}); leaves ctx tuned to the best."""
    results = {}
    t0 = time.time()
    for tile, block in itertools.product(tiles, blocks):
        try:
            ms = time_config(ctx, sid, cam, tile, block, frames=frames, animate=animate)
        except Exception as exc:  # a shape that does not fit (occupancy) is skipped
            if verbose:
                print(f"autotune: tile {tile} block {block} skipped: {exc}")
            continue
        results[(tile, block)] = ms
        if verbose:
            print(f"autotune: tile {tile:5d} block {block:3d}: {ms:.3f} ms/frame")
    best = min(results, key=results.get)
    ctx.set_tuning(tile_tris=best[0], block_threads=best[1])
    # second stage: the vertex chunk at the best tile and block
    chunk_ms = {}
    for ch in chunks:
        ctx.set_tuning(vertex_chunk=ch)
        chunk_ms[ch] = time_config(ctx, sid, cam, best[0], best[1], frames=frames, animate=animate)
        results[(best[0], best[1], ch)] = chunk_ms[ch]
        if verbose:
            print(f"autotune: tile {best[0]:5d} block {best[1]:3d} chunk {ch:5d}: {chunk_ms[ch]:.3f} ms/frame")
    bch = min(chunk_ms, key=chunk_ms.get)
    ctx.set_tuning(vertex_chunk=bch)
    best = (best[0], best[1], bch)
    if verbose:
        print(f"autotune: best {best} in {time.time() - t0:.1f} s")
    return best, results
