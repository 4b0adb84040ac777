"""Launch-shape autotuner for the kinetic step of a mesh or batch.

The step kernel is a cooperative persistent kernel; three knobs change its
speed but never its result:

* blocks per SM of the cooperative grid (occupancy against per-block latency
  of the grid-wide barriers of the flip rounds);
* the work-list size at or below which a single block finishes the flip rounds
  (block barriers instead of grid barriers for the long tail of small rounds);
* the removal tile: how many lanes of a warp take entries of the repair's
  vertex lists (its removals are long divergent chains).

The first two are searched jointly, then the tile at the best pair.  Each
candidate runs on a fresh clone of the mesh, so every candidate steps the same
state with the same displacement stream; the fastest (median of the timed
steps, CUDA events on the launching stream) is applied to the mesh.
"""
import itertools

import numpy as np


def _time(mesh, one_step, setting, warm, steps, stream):
    import torch

    m = mesh.clone()
    try:
        m.set_tuning(setting["blocks_per_sm"], setting["tail_items"], setting["removal_tile"])
        for k in range(warm):
            one_step(m, k, stream)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            ev[k][0].record(stream)
            one_step(m, warm + k, stream)
            ev[k][1].record(stream)
        stream.synchronize()
        ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
        st = m.status(stream)
        if st["status"] != 0:
            raise RuntimeError(f"autotune candidate failed: {st}")
    finally:
        m.close()
    return dict(setting, ms=ms)


def autotune(mesh, one_step, blocks=None, tails=(256, 1024, 2048, 8192), tiles=(0, 1, 4, 32), warm=1, steps=3,
             stream=None):
    """``one_step(m, k, stream)`` launches step k of the workload on mesh ``m`` (a
    MeshBatch); returns (best dict, list of all timings)."""
    import torch

    stream = stream or torch.cuda.current_stream()
    mx = mesh.tuning()["max_blocks_per_sm"]
    blocks = [b for b in (blocks or range(1, mx + 1)) if b <= mx]
    results = [_time(mesh, one_step, dict(blocks_per_sm=bps, tail_items=tail, removal_tile=0), warm, steps, stream)
               for bps, tail in itertools.product(blocks, tails)]
    best = min(results, key=lambda r: r["ms"])
    for tile in tiles:
        if tile == 0:
            continue
        results.append(_time(mesh, one_step, dict(best, removal_tile=tile), warm, steps, stream))
    best = min(results, key=lambda r: r["ms"])
    mesh.set_tuning(best["blocks_per_sm"], best["tail_items"], best["removal_tile"])
    return best, results
