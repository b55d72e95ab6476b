"""Launch-shape autotuner of the batched form.

A batched cycle can run with different launch shapes -- tile width (work items
per tile = threads per block), fusion depth (the x and y launches of a stage
separate, or fused into one launch) and the number of blocks of each persistent
launch.  Results never depend on the shape; speed does, a little, with the
instance sizes.  ``tune_batch`` times each candidate on the batch's own initial
state, keeps the fastest, re-uploads the initial state, and caches the choice
per (device, batch geometry, method) in a JSON file.
"""
from __future__ import annotations

import hashlib
import json
import os
import time

CACHE = os.path.join(os.environ.get("XDG_CACHE_HOME", os.path.expanduser("~/.cache")), "pythonmhd_gb300",
                     "batch_tuning.json")


def _device():
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return p.name, p.multi_processor_count


def _key(batch, recon, name):
    shapes = ",".join(f"{a}x{b}" for a, b in batch.shapes)
    h = hashlib.sha1(shapes.encode()).hexdigest()[:16]
    return f"{name}|n={batch.count}|shapes={h}|mhd={batch.mhd}|recon={recon}|arith={batch.arith}"


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(table):
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE + ".tmp", "w") as f:
            json.dump(table, f, indent=1)
        os.replace(CACHE + ".tmp", CACHE)
    except OSError:
        pass


def _upload_all(batch, states):
    for k, st in enumerate(states):
        if batch.mhd:
            batch.upload(k, st["prim"], st["cons"], st["fbx"], st["fby"])
        else:
            batch.upload(k, st["prim"], st["cons"])


def tune_batch(batch, states, recon, cfl=0.4, cycles=2, use_cache=True,
               widths=(64, 128), fusions=(1, 2), blocks_per_sm=(2, 4)):
    """Pick and apply the fastest launch shape for ``batch``; returns the record."""
    import torch
    name, sms = _device()
    key = _key(batch, recon, name)
    table = _load() if use_cache else {}
    if key in table:
        rec = table[key]
        batch.configure(rec["tile_width"], rec["fuse"], rec["blocks"])
        return dict(rec, cached=True)
    trials = []
    for tw in widths:
        for fu in fusions:
            for bps in blocks_per_sm:
                batch.configure(tw, fu, bps * sms)
                _upload_all(batch, states)
                batch.advance(0.0, 1e30, 0, 1, cfl)          # builds the graph
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                batch.advance(0.0, 1e30, 1, 1 + cycles, cfl)
                torch.cuda.synchronize()
                trials.append((time.perf_counter() - t0, tw, fu, bps * sms))
    trials.sort()
    best = trials[0]
    rec = {"tile_width": best[1], "fuse": best[2], "blocks": best[3], "seconds_per_cycle": best[0] / cycles,
           "trials": [{"tile_width": t[1], "fuse": t[2], "blocks": t[3], "seconds_per_cycle": t[0] / cycles}
                      for t in trials]}
    batch.configure(best[1], best[2], best[3])
    _upload_all(batch, states)
    if use_cache:
        table[key] = rec
        _store(table)
    return dict(rec, cached=False)
