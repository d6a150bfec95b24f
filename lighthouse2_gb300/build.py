"""In-tree build of the GB300 render core: nvcc for sm_103a, one shared library.

    python -m lighthouse2_gb300.build        # -> lighthouse2_gb300/_build/libRenderCore_GB300.so
    LH2G_NVCC_FLAGS="-DLH2G_COOP=1" python -m lighthouse2_gb300.build -f   # another traversal strategy

The library exports the C ABI of include/lh2g.h and the Lighthouse 2 plugin entry point CreateCore
(include/lh2_core_api.h). Device code is compiled without fast-math and with --fmad=false: the shading
arithmetic must round exactly like its IEEE single-precision statement (explicit fmaf calls in culling code
are unaffected).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB_NAME = "libRenderCore_GB300.so"
LIB = os.path.join(OUT, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["bvh_build.cu", "kernels.cu", "adaptive.cu", "svgf.cu", "capi.cu", "rendercore.cu", "noalloc.cu", "server.cu", "nrc.cu", "raster.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _flags(defines=()):
    extra = os.environ.get("LH2G_NVCC_FLAGS", "").split()   # e.g. traversal strategy: -DLH2G_COOP=1 -DLH2G_REFILL=1
    return ARCH + extra + list(defines) + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                   "-Xcompiler", "-fPIC,-O2,-fvisibility=hidden,-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, out_dir=None, defines=()):
    """Compiles the library into out_dir (default lighthouse2_gb300/_build); `defines` are extra nvcc flags of a
    variant build (e.g. ["-DLH2G_STACK=12"] into its own directory), whose objects never mix with the default's."""
    out = out_dir or OUT
    lib = os.path.join(out, LIB_NAME)
    os.makedirs(out, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + _flags(defines) + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("nvcc failed for " + cmd[-3])
    if force or jobs or not os.path.exists(lib):
        link = [cc] + ARCH + ["-shared", "-o", lib + ".tmp"] + objs + ["-Xlinker", "--exclude-libs,ALL"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(link) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(lib + ".tmp", lib)
    return lib


HARNESS = os.path.join(OUT, "headless_app")


def build_harness(force=False):
    """The headless Lighthouse 2 application (harness/headless_app.cpp): host C++ only, loads a core by name."""
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "harness", "headless_app.cpp")
    deps = [src] + [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    if force or _stale(HARNESS, deps):
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
        cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, src, "-o", HARNESS + ".tmp", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("headless application build failed")
        os.replace(HARNESS + ".tmp", HARNESS)
    return HARNESS


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
    print(build_harness(force="-f" in sys.argv))
