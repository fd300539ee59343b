"""Build recipe for libgbtrace.so (the CUDA backend) for sm_103a.

Each .cu file is compiled to an object in trace_gb300/_build/ in parallel,
then linked into trace_gb300/libgbtrace.so.  No cmake, no torch: plain nvcc.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbtrace.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["api.cu", "lbvh.cu", "traverse.cu", "render.cu", "batch.cu", "adjoint.cu", "phr.cu", "collapse.cu", "heatmap.cu", "cost.cu",
           "noalloc.cu", "buffer.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "--expt-relaxed-constexpr"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps(src):
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)] + [src]


def _stale(out, inputs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in inputs)


def _extra():
    """Extra nvcc arguments from GBT_NVCC_EXTRA (e.g. "-DGBT_PT_DYN=12"), for measuring build
    variants; a change of them rebuilds every object."""
    return os.environ.get("GBT_NVCC_EXTRA", "").split()


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    stamp = os.path.join(BUILD, "extra_flags")
    if not _stale(obj, _deps(src) + ([stamp] if os.path.exists(stamp) else [])):
        return obj, ""
    cmd = [nvcc(), *ARCH, *FLAGS, *_extra(), "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose_ptxas=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "extra_flags")
    extra = " ".join(_extra())
    if (open(stamp).read() if os.path.exists(stamp) else "") != extra:
        with open(stamp, "w") as f:  # newer than every object: all are rebuilt with the new flags
            f.write(extra)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 1)) as ex:
        futs = {ex.submit(_compile, s, verbose_ptxas): s for s in srcs}
        objs = []
        for f in cf.as_completed(futs):
            o, log = f.result()
            objs.append(o)
            logs[os.path.basename(futs[f])] = log
    objs.sort()
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    for k, v in logs.items():
        if v.strip():
            print("==", k)
            print(v)
    print(lib)
