"""Autotuner of the batched mat-vec, with an on-disk cache.

The batched ensemble path (batch.Ensemble) has three mat-vec kernels for the
same product (the Kronecker contraction of field.py:1212-1243 in complex64):

* ``tensor``       tensor-core tiles (tcgen05, split TF32), A operands staged in
                   shared memory, R = 64 / KP rows x 128 vectors per tile;
* ``tensor_tmem``  the same products with the A operands written to tensor
                   memory and a deeper TMA ring of input rows;
* ``fp32``         every product an FP32 FMA, tiles of 128 / NKP rows x 32 vectors.

Which one is fastest depends on the operator's shape (slab sizes, K block
sizes, band widths) and on the number of vectors. ``choose`` times every
candidate on the operator (CUDA events, after one untimed launch) and keeps
the fastest; the choice is stored under a key made of the device name, the
operator's table shape (a hash of its slab, K-block and term tables, which
fixes every tile of every kernel), the vector block count and the precision,
in a JSON file (``$RICHMOL_GB300_TUNE_CACHE``, default
``~/.cache/richmol_gb300/matvec_tune.json``). A later ensemble of the same
shape reads the choice from the file and times nothing.
"""
import hashlib
import json
import os
import tempfile
import threading

import numpy as np

CACHE_ENV = "RICHMOL_GB300_TUNE_CACHE"
PRECISION = "c64-matvec/f64-lanczos"
_lock = threading.Lock()


def cache_path():
    p = os.environ.get(CACHE_ENV)
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "richmol_gb300", "matvec_tune.json")


def shape_key(plan, nvec, device_name):
    """Key of one tuning problem: device, operator table shape, vector blocks
    of 128, precision. The field (MF values) and K values do not enter: the
    kernels' tiles and loops depend on the tables' shapes only."""
    a = plan.tables.arrays
    h = hashlib.sha1()
    for name in ("out_dm", "out_dk", "in_dm", "in_dk", "k_rows", "k_cols", "k_type", "m_width", "t_out", "t_in",
                 "t_k", "t_mf", "mf_group", "out_stride", "in_stride"):
        if name in a:
            h.update(name.encode())
            h.update(np.ascontiguousarray(a[name]).tobytes())
    nblk = (int(nvec) + 127) // 128
    return f"{device_name}|dim={plan.dim_out}|terms={plan.nterm}|tables={h.hexdigest()[:16]}|vblocks={nblk}|{PRECISION}"


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store_choice(key, kind, times, path=None):
    """Adds one entry to the cache file (read, update, atomic replace)."""
    path = path or cache_path()
    with _lock:
        data = load_cache(path)
        data[key] = {"kind": kind, "ms": {k: round(float(v), 4) for k, v in times.items()}}
        d = os.path.dirname(path) or "."
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=d, prefix=".tune", suffix=".json")
        with os.fdopen(fd, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def lookup(key, kinds, path=None):
    e = load_cache(path).get(key)
    if isinstance(e, dict) and e.get("kind") in kinds:
        return e["kind"], e.get("ms", {})
    return None


def time_kinds(run, kinds, reps=3):
    """ms per call of run(kind) for every kind (CUDA events around reps calls,
    after one untimed call)."""
    import torch
    times = {}
    for k in kinds:
        run(k)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            run(k)
        b.record()
        b.synchronize()
        times[k] = a.elapsed_time(b) / reps
    return times


def choose(plan, nvec, kinds, run, device_name, use_cache=True, path=None, reps=3, timer=None):
    """The fastest kind for this operator shape and vector count: from the
    cache when present, else timed (run(kind) launches one mat-vec of that
    kind; timer(run, kinds, reps) -> ms per kind, default time_kinds) and
    stored. Returns (kind, ms per kind, from_cache)."""
    key = shape_key(plan, nvec, device_name)
    if use_cache:
        hit = lookup(key, kinds, path)
        if hit is not None:
            return hit[0], hit[1], True
    times = (timer or time_kinds)(run, kinds, reps)
    best = min(times, key=times.get)
    if use_cache:
        store_choice(key, best, times, path)
    return best, times, False
