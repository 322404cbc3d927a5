"""C++ operator layer on the CPU: exports, the plan runner and its libconfig
parser over memscan leaves, refused plans, the Error a GPU operator must
return without a GPU, and the same operator source linked into the reference
engine's own Query (when the reference tree was built here)."""
import os
import subprocess

import numpy as np
import pytest

from pythia_gb300 import plans

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCAN = '''
buffsize = 48;   # three 16-byte tuples per page
treeroot = { name = "scan"; };
scan = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
'''

JOIN = '''
buffsize = 64;
treeroot = { name = "join"; build = { name = "r"; }; probe = { name = "s"; }; };
r = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
s = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
join = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("P$1", "B$1");
         threadgroups = ((0, 1)); hash = { fn = "modulo"; buckets = 64; }; tuplesperbucket = 4; };
'''


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_library_exports_runner_and_operator_classes():
    syms = _exports(plans.lib_path())
    assert {"pgo_register", "pgo_run", "pgo_free"} <= syms
    for cls in ("GpuHashJoinOp", "GpuMPSMJoinOp", "GpuPartitionOp", "GpuAggregateSumOp", "GpuAggregateCountOp"):
        assert f"_ZTIN14pythia_gpu_ops{len(cls)}{cls}E" in syms, cls


def test_memscan_threads_read_consecutive_slices():
    R = np.arange(40, dtype=np.int64).reshape(20, 2)
    plans.register("R", R)
    for threads in (1, 3, 7):
        rows, per = plans.run(SCAN, threads=threads)
        assert per == [20 * (t + 1) // threads - 20 * t // threads for t in range(threads)]
        assert np.array_equal(rows.view(np.int64).reshape(-1, 2), R)


def test_parser_accepts_libconfig_forms():
    R = np.arange(8, dtype=np.int64).reshape(4, 2)
    plans.register("R2", R)
    plan = '''
    /* block comment */ buffsize : 0x10L;      // 16 bytes, hex with L suffix
    treeroot = { name = "sc" "an"; };           # adjacent strings concatenate
    scan = { type = "memscan"; relation = "R2"; schema = [ "LONG", "long" ]; extra = { a = 1.5e0; b = true; c = (); }; };
    '''
    rows, per = plans.run(plan, threads=2)
    assert per == [2, 2]
    assert np.array_equal(rows.view(np.int64).reshape(-1, 2), R)


@pytest.mark.parametrize("plan,needle", [
    ('treeroot = { name = "x"; }; x = { type = "nope"; };', "not a GPU operator type"),
    ('treeroot = { name = ', "expected a value"),
    (JOIN.replace('"P$1"', '"X$1"'), "bad projection"),
    (JOIN.replace('"P$1"', '"P$7"'), "out of range"),
    (JOIN.replace('relation = "R"; schema = ("long", "long"); };\njoin',
                  'relation = "R"; schema = ("long", "dec"); };\njoin').replace("probejattr = 0", "probejattr = 1"),
     "integer join keys"),
    (SCAN.replace('"R"', '"missing"'), "not registered"),
    (SCAN.replace('("long", "long")', '("long", "int")'), "width mismatch"),
])
def test_refused_plans(plan, needle):
    plans.register("R", np.arange(40, dtype=np.int64).reshape(20, 2))
    with pytest.raises(plans.PlanError) as e:
        plans.run(plan, threads=2)
    assert e.value.code == 2 and needle in str(e.value)


def test_gpu_operator_without_gpu_returns_error():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    plans.register("R", np.arange(40, dtype=np.int64).reshape(20, 2))
    with pytest.raises(plans.PlanError) as e:
        plans.run(JOIN, threads=2)
    assert e.value.code == 1


def test_phase_trace_records_operator_threads():
    # The trace names the plan node, the thread and the phase; each of the
    # group's two threads starts, and its first thread launches once, even
    # when the launch fails for want of a GPU. Off, nothing is recorded.
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    plans.register("R", np.arange(40, dtype=np.int64).reshape(20, 2))
    plans.trace(True)
    try:
        with pytest.raises(plans.PlanError):
            plans.run(JOIN, threads=2)
        t = plans.trace_read()
    finally:
        plans.trace(False)
    assert sorted((node, tid) for _, node, tid, ph in t if ph == "start") == [("join", 0), ("join", 1)]
    assert [(node, tid) for _, node, tid, ph in t if ph == "launch"] == [("join", 0)]
    assert [ph for _, _, tid, ph in t if tid == 0][-2:] == ["launch", "done"]
    for tid in (0, 1):
        ns = [e[0] for e in t if e[2] == tid]
        assert ns == sorted(ns)
    with pytest.raises(plans.PlanError):
        plans.run(JOIN, threads=2)
    assert plans.trace_read() == t                                     # off: nothing added


def test_gpu_chain_without_gpu_returns_error_and_moves_nothing():
    # partition -> join with the device exchange set up at init: without a GPU
    # the partition fails in scanStart, the join sees its child's Error, every
    # thread returns Error and no bytes are counted as moved.
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    plans.register("R", np.arange(40, dtype=np.int64).reshape(20, 2))
    plan = """
    buffsize = 4096;
    treeroot = { name = "join"; build = { name = "pr"; input = { name = "r"; }; };
                                probe = { name = "ps"; input = { name = "s"; }; }; };
    r = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
    s = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
    pr = { type = "gpupartition"; attr = 0; range = (0, 39); buckets = 2; };
    ps = { type = "gpupartition"; attr = 0; range = (0, 39); buckets = 2; };
    join = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("P$1", "B$1");
             threadgroups = ((0), (1)); };
    """
    plans.transfer_stats(reset=True)
    for on in (True, False):
        plans.set_device_exchange(on)
        try:
            with pytest.raises(plans.PlanError) as e:
                plans.run(plan, threads=2)
        finally:
            plans.set_device_exchange(True)
        assert e.value.code == 1
    assert plans.transfer_stats() == {"h2d": 0, "d2h": 0, "d2d": 0, "in_place": 0, "direct": 0}


def test_reference_engine_drives_gpu_operator():
    # The engine's own Query::create, with this repository's plan factory in
    # place of query.o, builds hashjoin, gpuhashjoin, gpumpsmjoin and
    # gpuaggregate_count plans (the GPU joins are dual-input types the engine
    # cannot take as user-defined operators); the CPU join must give the
    # engine's answer and every GPU plan must be constructed and initialised.
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_gpuops_check")
    if not os.path.exists(exe):
        pytest.skip("reference engine not built here")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    for name in ("hashjoin:", "gpuhashjoin:", "gpumpsmjoin:", "gpuaggregate_count:"):
        assert any(ln.startswith(name) and ln.endswith("ok") for ln in r.stdout.splitlines()), r.stdout
