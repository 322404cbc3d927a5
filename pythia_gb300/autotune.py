"""Launch-shape autotuner for the GPU operators.

Sweeps, per size class, the knobs that change speed but never results:

* batched joins (pg_batch_*): threads per CTA, probe keys in flight per
  thread, tile size, persistent CTAs per SM and table load factor (bucket
  size), separately for small / medium / large instances;
* the page sort's radix digit: 4..12 bits, i.e. partition fan-out 2^bits;
* the partition tile size and the hash-join probe's CTAs per SM.

Results are cached as JSON (pythia_gb300/.autotune.json by default) keyed by
GPU name, so later runs reuse them.
"""
import ctypes
import json
import os
import time  # noqa: F401  (time_batch)

from pythia_gb300 import gpu

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), ".autotune.json")

SIZE_CLASSES = (("small", 0, 16 << 10), ("medium", 16 << 10, 512 << 10), ("large", 512 << 10, 1 << 62))

BATCH_SHAPES = [
    dict(threads=t, items=i, tile=tl, ctas_per_sm=c, load_inverse=li, use_graph=1)
    for t, i, tl, c, li in [
        (256, 4, 4096, 4, 2), (256, 8, 4096, 4, 2), (512, 4, 4096, 2, 2), (128, 4, 1024, 8, 2),
        (256, 4, 1024, 8, 2), (256, 4, 16384, 4, 2), (256, 2, 4096, 8, 2), (256, 4, 4096, 4, 4),
        (512, 8, 16384, 2, 2), (128, 8, 2048, 8, 4),
    ]
]


def size_class(n_build):
    for name, lo, hi in SIZE_CLASSES:
        if lo <= n_build < hi:
            return name
    return "large"


def shape_struct(d):
    return gpu.BatchShape(d["threads"], d["items"], d["tile"], d["ctas_per_sm"], d["load_inverse"],
                          d.get("use_graph", 1))


def prepare(ctx, items, shape):
    arr = (gpu.BatchItem * max(1, len(items)))()
    for k, (R, nR, S, nS) in enumerate(items):
        arr[k] = gpu.BatchItem(R, nR, S, nS)
    b = ctypes.c_void_p()
    sh = shape_struct(shape)
    ctx._check(gpu.lib().pg_batch_prepare(ctx.h, ctx.stream, arr, len(items), ctypes.byref(sh), ctypes.byref(b)))
    return b.value


def run(ctx, b, counts=None):
    ctx._check(gpu.lib().pg_batch_run(ctx.h, b, counts.ctypes.data if counts is not None else None))


def free(ctx, b):
    gpu.lib().pg_batch_free(ctx.h, b)


def time_batch(ctx, b, repeats=3):
    run(ctx, b)
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        run(ctx, b)
        best = min(best, time.perf_counter() - t0)
    return best


def tune_batch(ctx, items_by_class, shapes=BATCH_SHAPES, repeats=3, log=None):
    """items_by_class: {class: [(R_ptr, nR, S_ptr, nS), ...]}. Times every
    shape per class in the library (pg_autotune_batch, CUDA events) and
    returns the fastest shape per class and the sweep table."""
    best, table = {}, {}
    arr_shapes = (gpu.BatchShape * len(shapes))(*[shape_struct(sh) for sh in shapes])
    for cls, items in items_by_class.items():
        if not items:
            continue
        arr = (gpu.BatchItem * len(items))(*[gpu.BatchItem(R, nR, S, nS) for (R, nR, S, nS) in items])
        pick = ctypes.c_uint32()
        ms = (ctypes.c_double * len(shapes))()
        ctx._check(gpu.lib().pg_autotune_batch(ctx.h, ctx.stream, arr, len(items), arr_shapes, len(shapes),
                                               repeats, ctypes.byref(pick), ms))
        rows = sorted(((ms[k], shapes[k]) for k in range(len(shapes))), key=lambda r: r[0])
        if log:
            for t, sh in rows:
                log(f"{cls} {sh} {t:.3f} ms")
        best[cls] = shapes[pick.value]
        table[cls] = [{"ms": t, **sh} for t, sh in rows]
    return best, table


def load(gpu_name):
    if os.path.exists(CACHE):
        try:
            return json.load(open(CACHE)).get(gpu_name)
        except (OSError, ValueError):
            return None
    return None


def save(gpu_name, entry):
    data = {}
    if os.path.exists(CACHE):
        try:
            data = json.load(open(CACHE))
        except (OSError, ValueError):
            data = {}
    data[gpu_name] = entry
    with open(CACHE, "w") as f:
        json.dump(data, f, indent=1)
