"""Build recipe for the native parts of pythia_gb300 (no cmake, no setuptools).

  libpythia_gpu.so        CUDA kernels + C ABI (include/pythia_gpu.h), sm_103a
  libpythia_gpuops.so     C++ operator layer (Gpu*Op) over the C ABI
  libpythia_datagen.so    seeded synthetic relations (C)

Translation units compile in parallel; objects go to pythia_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
GPUOPS = os.path.join(PKG, "gpuops")
BUILD = os.path.join(PKG, "_build")
GENCODE = "arch=compute_103a,code=sm_103a"

CU_SOURCES = ["pg_core.cu", "pg_partition.cu", "pg_hashjoin.cu", "pg_groupby.cu",
              "pg_sort.cu", "pg_mpsm.cu", "pg_batch.cu", "pg_noalloc.cu", "pg_htimage.cu", "pg_filter.cu"]
NVCC_FLAGS = ["-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17",
              "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-O3",
              "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=cwd)
    if r.returncode:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers():
    hs = [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
    hs += [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    return hs


def build_gpu(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    srcs = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []

    def one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        path = os.path.join(CSRC, src)
        if _stale(obj, [path] + hdrs):
            out = _run([nvcc] + NVCC_FLAGS + ["-Xptxas", "-v", "-c", path, "-o", obj])
            if verbose:
                print(out)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, srcs))
    lib = os.path.join(PKG, "libpythia_gpu.so")
    if _stale(lib, objs):
        _run([nvcc, "-shared", "-gencode", GENCODE, "-o", lib] + objs + ["-lcudart"])
    return lib


def build_datagen():
    src = os.path.join(PKG, "datagen", "datagen.c")
    lib = os.path.join(PKG, "datagen", "libpythia_datagen.so")
    if _stale(lib, [src]):
        _run(["gcc", "-O3", "-fPIC", "-shared", "-Wall", src, "-o", lib, "-lpthread", "-lm"])
    return lib


def build_host():
    """C++ operator layer (Gpu*Op classes, gpuops/) on the mirror of the
    engine's operator interface, with the plan runner, linked against
    libpythia_gpu.so. C++98 like the engine, so the same operator source also
    compiles against the engine's own headers (oracle/Makefile.ref)."""
    srcs = [os.path.join(GPUOPS, "mirror", "pythia_mirror.cpp"), os.path.join(GPUOPS, "gpuops.cpp"),
            os.path.join(GPUOPS, "harness.cpp")]
    lib = os.path.join(PKG, "libpythia_gpuops.so")
    deps = srcs + [os.path.join(GPUOPS, "gpuops.h"), os.path.join(GPUOPS, "mirror", "pythia_mirror.h")]
    deps += _headers() + [os.path.join(PKG, "libpythia_gpu.so")]
    if _stale(lib, deps):
        _run(["g++", "-O2", "-std=gnu++98", "-fPIC", "-shared", "-pthread", "-Wall", "-Wno-unused-parameter",
              "-I" + os.path.join(ROOT, "include"), "-I" + GPUOPS] + srcs +
             ["-L" + PKG, "-lpythia_gpu", "-Wl,-rpath,$ORIGIN", "-o", lib])
    return lib


def build_oracle(reference=None):
    """The C oracle (test infrastructure) and, when `reference` (or the
    PYTHIA_REFERENCE environment variable) names the reference source tree and
    it is present, the reference engine itself (oracle/Makefile.ref)."""
    src = os.path.join(ROOT, "oracle", "pythia_oracle.c")
    lib = os.path.join(ROOT, "oracle", "liboracle.so")
    if _stale(lib, [src, os.path.join(ROOT, "oracle", "pythia_oracle.h")]):
        _run(["gcc", "-O3", "-fPIC", "-shared", "-Wall", src, "-o", lib, "-lpthread", "-lm"])
    ref = reference or os.environ.get("PYTHIA_REFERENCE")
    if ref and os.path.isdir(ref) and os.path.exists(os.path.join(ref, "operators", "join.cpp")):
        _run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"),
              "REF=" + ref, "-j", str(min(8, os.cpu_count() or 4))], cwd=ROOT)
    return lib


def build_all(verbose=False, reference=None):
    build_datagen()
    build_gpu(verbose=verbose)
    build_host()
    build_oracle(reference)     # after libpythia_gpu: the reference build links the operators against it


if __name__ == "__main__":
    build_all(verbose=True)
