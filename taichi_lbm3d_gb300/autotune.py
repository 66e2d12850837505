"""Autotuner for the batched persistent kernel.

For each subvolume edge size it times the persistent step kernel over a small
batch of subvolumes of that size for every candidate (work-tile length, CTA
size), with CUDA events on the batch's stream, and keeps the fastest.  Results
are cached in a JSON file keyed by GPU name, storage mode and edge size
(default ``~/.cache/taichi_lbm3d_gb300/autotune.json``, or $LBM_AUTOTUNE_CACHE),
so a later run with the same key does not time again.
"""
import json
import os
import time

import numpy as np

TILES = (256, 512, 1024, 2048, 4096)
BLOCKS = (128, 256)


def cache_path():
    return os.environ.get("LBM_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "taichi_lbm3d_gb300", "autotune.json"))


def _load(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _save(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def time_config(batch, tile, block, steps=20, warmup=4):
    """Seconds per step of the persistent kernel with (tile, block)."""
    import torch
    batch.configure([tile] * batch.n, block)
    batch.init()
    batch.step(warmup, chunk=warmup)
    stream = torch.cuda.ExternalStream(batch.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    batch.step(steps, chunk=steps)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / steps


def tune(solids_by_edge, storage="f16", force=(1e-6, 0, 0), niu=0.1, path=None, retune=False, log=None):
    """solids_by_edge: {edge: [solid masks of that edge]}.  Returns
    {edge: {"tile": t, "block": b, "ms_per_step": ...}} and updates the cache."""
    from .batch import Batch
    path = path or cache_path()
    cache = _load(path)
    gpu = _gpu_name()
    out = {}
    for edge, solids in sorted(solids_by_edge.items()):
        key = "%s|%s|%d" % (gpu, storage, edge)
        if key in cache and not retune:
            out[edge] = cache[key]
            continue
        b = Batch(solids, niu=niu, force=force, storage=storage)
        best = None
        trials = {}
        for block in BLOCKS:
            for tile in TILES:
                t = time_config(b, tile, block)
                trials["%d/%d" % (tile, block)] = t * 1e3
                if best is None or t < best[0]:
                    best = (t, tile, block)
        nf = b.info()["n_fluid"]
        b.close()
        res = {"tile": best[1], "block": best[2], "ms_per_step": best[0] * 1e3,
               "mlups": nf / best[0] / 1e6, "trials_ms": trials, "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
        cache[key] = res
        out[edge] = res
        if log:
            log("autotune edge %d: tile %d block %d (%.3f ms/step, %.0f MLUPS)" % (edge, best[1], best[2],
                                                                                 best[0] * 1e3, res["mlups"]))
    _save(path, cache)
    return out


def plan(edges, tuned):
    """Per-subvolume tile lengths and one CTA size for a mixed batch: each
    subvolume uses its edge's tile length; the CTA size is the one tuned for
    the edge class holding the most cells."""
    tiles = [int(tuned[e]["tile"]) for e in edges]
    weight = {}
    for e in edges:
        weight[e] = weight.get(e, 0) + e ** 3
    heavy = max(weight, key=weight.get)
    return tiles, int(tuned[heavy]["block"])
