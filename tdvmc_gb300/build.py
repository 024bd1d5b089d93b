"""Build the in-tree CUDA library (sm_103a) and the native host driver.

    python -m tdvmc_gb300.build

Outputs (git-ignored): tdvmc_gb300/_lib/libtdvmc_gb300.so and
tdvmc_gb300/_lib/tdvmc_run.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libtdvmc_gb300.so")
RUNNER = os.path.join(LIBDIR, "tdvmc_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation units compiled in parallel; the kernel instantiations are
# spread over them by the TDVMC_TU_* macros in tdvmc_capi.cu
UNITS = ["tdvmc_capi.cu", "inst_sample_f32.cu", "inst_sample_f64.cu", "inst_eloc_f32.cu", "inst_eloc_f64.cu", "inst_pb.cu",
         "k_gram_tf32.cu", "k_peak.cu", "noalloc_stats.cu", "drops_capi.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, u) for u in UNITS]


def _deps():
    out = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                out.append(os.path.join(d, f))
    out.append(os.path.abspath(__file__))
    return out


def _stale(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale(LIB):
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    nv = nvcc()
    flags = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]
    if verbose:
        flags += ["-Xptxas", "-v"]

    def comp(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        r = subprocess.run([nv, *flags, "-dc" if False else "-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(UNITS), os.cpu_count() or 4))) as ex:
        results = list(ex.map(comp, _sources()))
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call([nv, *ARCH, "-shared", "--cudart", "shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    build_runner()
    return LIB


def build_runner() -> str:
    """Native host driver (C++17) over the C ABI: config / time loop / output files."""
    src = os.path.join(CSRC, "host", "tdvmc_run.cpp")
    if not os.path.exists(src):
        return ""
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), src, "-o", RUNNER,
           "-L" + LIBDIR, "-ltdvmc_gb300", "-Wl,-rpath,$ORIGIN"]
    subprocess.check_call(cmd)
    return RUNNER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
