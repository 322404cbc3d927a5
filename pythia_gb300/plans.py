"""Pythia plans with GPU operators, run through the C++ operator layer.

The plan is libconfig text as the engine reads it: `buffsize`, `treeroot`
naming the root node, one top-level group per node with its `type` and keys,
`input` (single-input) or `build` / `probe` (dual-input) naming children. GPU
operator types: gpuhashjoin, gpumpsmjoin, gpupartition, gpuaggregate_sum,
gpuaggregate_count (libpythia_gpuops, pythia_gb300/gpuops/). Leaves are
`memscan` nodes over relations registered from numpy arrays: thread t of T
reads rows [t n / T, (t + 1) n / T).

    plans.register("R", R)                 # (n, width) uint8 / int64 rows
    out, per_thread = plans.run(PLAN, threads=4)

`run` returns every thread's output tuples in thread order as one
(rows, tuple_size) uint8 array and the per-thread row counts. An operator
that returns Error (a GPU failure, or no GPU at all: there is no CPU path)
raises PlanError with code 1; a plan the operators refuse raises code 2.
"""
import ctypes
import os

import numpy as np

_LIB = None
_KEEP = {}          # registered arrays stay alive while plans may read them


class PlanError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"plan failed ({code}): {msg}")
        self.code = code


def lib_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "libpythia_gpuops.so")


def lib():
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(path)
        L.pgo_register.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_uint]
        L.pgo_register.restype = ctypes.c_int
        L.pgo_run.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                              ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_uint),
                              ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_char_p, ctypes.c_int]
        L.pgo_run.restype = ctypes.c_int
        L.pgo_free.argtypes = [ctypes.c_void_p]
        L.pgo_free.restype = None
        L.pgo_transfer_stats.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)]
        L.pgo_transfer_stats.restype = None
        L.pgo_reset_transfer_stats.argtypes = []
        L.pgo_reset_transfer_stats.restype = None
        L.pgo_set_device_exchange.argtypes = [ctypes.c_int]
        L.pgo_set_device_exchange.restype = None
        L.pgo_pin.argtypes = [ctypes.c_char_p, ctypes.c_int]
        L.pgo_pin.restype = ctypes.c_int
        L.pgo_trace.argtypes = [ctypes.c_int]
        L.pgo_trace.restype = None
        L.pgo_trace_dump.argtypes = [ctypes.c_char_p, ctypes.c_ulonglong]
        L.pgo_trace_dump.restype = ctypes.c_ulonglong
        _LIB = L
    return _LIB


_PINNED = set()


def register(name, rows, pin=False):
    """Makes `rows` (a C-contiguous 2-D array, one row per tuple) readable by
    memscan nodes with `relation = name`. pin=True page-locks its memory (a
    loader reading into pinned memory): GPU operators then copy its pages to
    the device directly instead of through staging buffers."""
    a = np.ascontiguousarray(rows)
    if a.ndim != 2:
        raise ValueError("rows must be 2-D")
    width = a.shape[1] * a.itemsize
    if name in _PINNED:
        lib().pgo_pin(name.encode(), 0)
        _PINNED.discard(name)
    _KEEP[name] = a
    if lib().pgo_register(name.encode(), a.ctypes.data if a.size else None, a.shape[0], width):
        raise ValueError("pgo_register refused the relation")
    if pin and a.size:
        if lib().pgo_pin(name.encode(), 1):
            raise RuntimeError("pgo_pin failed (no GPU, or the memory could not be page-locked)")
        _PINNED.add(name)


def run(plan, threads=1):
    out = ctypes.c_void_p()
    nbytes = ctypes.c_ulonglong()
    tsize = ctypes.c_uint()
    per = (ctypes.c_ulonglong * threads)()
    err = ctypes.create_string_buffer(1024)
    rc = lib().pgo_run(plan.encode(), threads, ctypes.byref(out), ctypes.byref(nbytes), ctypes.byref(tsize),
                       per, err, len(err))
    try:
        if rc:
            raise PlanError(rc, err.value.decode(errors="replace"))
        w = tsize.value
        buf = np.frombuffer(ctypes.string_at(out.value, nbytes.value), dtype=np.uint8).copy() \
            if nbytes.value else np.zeros(0, np.uint8)
        rows = buf.reshape(-1, w) if w else buf.reshape(0, 0)
        return rows, [int(per[t]) // max(w, 1) for t in range(threads)]
    finally:
        if out.value:
            lib().pgo_free(out)


def transfer_stats(reset=False):
    """Bytes the GPU operators moved since the last reset: pages uploaded
    ("h2d"), outputs downloaded ("d2h"), device copies gathering inputs
    ("d2d"), inputs taken on the device in place ("in_place", a count), and
    the part of "h2d" copied straight from pinned or registered pages ("direct")."""
    a = (ctypes.c_ulonglong * 5)()
    lib().pgo_transfer_stats(a)
    if reset:
        lib().pgo_reset_transfer_stats()
    return {"h2d": a[0], "d2h": a[1], "d2d": a[2], "in_place": a[3], "direct": a[4]}


def trace(on=True):
    """Turns the GPU operators' phase trace on (emptying it) or off."""
    lib().pgo_trace(1 if on else 0)


def trace_read():
    """The phase trace as (ns, node, thread, phase) tuples in arrival order:
    host monotonic nanoseconds, the plan node of the operator, the operator
    thread and the phase it reached."""
    need = lib().pgo_trace_dump(None, 0)
    buf = ctypes.create_string_buffer(int(need))
    lib().pgo_trace_dump(buf, need)
    out = []
    for line in buf.value.decode().splitlines():
        ns, node, tid, phase = line.split(" ", 3)
        out.append((int(ns), node, int(tid), phase))
    return out


def set_device_exchange(on):
    """Adjacent GPU operators keep their data on the device (default True);
    False makes every operator read and write host pages."""
    lib().pgo_set_device_exchange(1 if on else 0)
