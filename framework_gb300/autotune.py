"""Brick-shape autotuner for batched extraction.

The brick sweep covers 128 columns x 32 rows x P z-planes per unit of the
persistent work queue.  Long bricks amortise the z halo plane; short bricks
give more queue entries to balance uneven batches across the 152 SMs.  The
best P depends on the mix of volume sizes, so it is measured: each candidate
runs the batch a few times (graph mode, CUDA events) and the fastest wins.

Results persist in a JSON file keyed by the device name and a signature of
the batch (volume count, dtype mix, log2 histogram of cell counts), so a
service pays the tuning cost once per workload shape.
"""
import json
import math
import os

CANDIDATES = (0, 2, 4, 8, 16, 32)   # 0: the library's own choice from the batch size
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def batch_signature(volumes):
    """Shape signature of a batch: count, dtypes, histogram of log2(cells)."""
    hist = {}
    dtypes = set()
    for d in volumes:
        t = d["volume"]
        nz, ny, nx = t.shape
        cells = max(nx - 1, 0) * max(ny - 1, 0) * max(nz - 1, 0)
        b = int(math.log2(cells)) if cells > 0 else -1
        hist[b] = hist.get(b, 0) + 1
        dtypes.add(str(t.dtype).replace("torch.", ""))
    h = ",".join("%d:%d" % (k, hist[k]) for k in sorted(hist))
    return "n=%d;dt=%s;h=%s" % (len(volumes), "+".join(sorted(dtypes)), h)


def _device_key(device):
    import torch
    p = torch.cuda.get_device_properties(device)
    return "%s/sm%d" % (p.name, p.multi_processor_count)


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = "%s.%d.tmp" % (path, os.getpid())   # ranks of one job may save at the same time
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def time_batch(ex, volumes, vertices, quads, triangles=None, reps=3):
    """Mean device milliseconds of one graph-mode batch (after one warm-up)."""
    import torch
    stream = torch.cuda.current_stream()
    ex.extract_batch(volumes, vertices, quads, triangles, mode="graph", stream=stream)
    ex.batch_wait()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total = 0.0
    for _ in range(reps):
        e0.record(stream)
        ex.extract_batch(volumes, vertices, quads, triangles, mode="graph", stream=stream)
        e1.record(stream)
        ex.batch_wait()
        e1.synchronize()
        total += e0.elapsed_time(e1)
    return total / reps


def tune(ex, volumes, vertices, quads, triangles=None, candidates=CANDIDATES, reps=3, cache=DEFAULT_CACHE,
         force=False):
    """Choose the planes-per-brick option for this batch shape and apply it
    to ``ex``.  Returns {"planes": P, "ms": {P: ms, ...}, "cached": bool}."""
    from . import OPT_BRICK_PLANES
    key = _device_key(ex.device) + "|" + batch_signature(volumes)
    data = _load(cache) if cache else {}
    if not force and key in data:
        ex.set_option(OPT_BRICK_PLANES, int(data[key]["planes"]))
        return dict(data[key], cached=True)
    timings = {}
    for p in candidates:
        ex.set_option(OPT_BRICK_PLANES, int(p))
        timings[int(p)] = time_batch(ex, volumes, vertices, quads, triangles, reps)
    best = min(timings, key=timings.get)
    ex.set_option(OPT_BRICK_PLANES, best)
    entry = {"planes": best, "ms": {str(k): round(v, 4) for k, v in timings.items()}}
    if cache:
        data[key] = entry
        _save(cache, data)
    return dict(entry, cached=False)
