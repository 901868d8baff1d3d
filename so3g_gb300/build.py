"""Build the GB300 CUDA library (libso3g_gb300.so) in-tree.

Each translation unit under csrc/ is compiled by nvcc for sm_103a only, in
parallel, and linked into so3g_gb300/_lib/libso3g_gb300.so with the CUDA
runtime linked statically.  All units are compiled with ``-fmad=false`` so
that no multiply-add is fused anywhere: the float64 pointing arithmetic
then rounds exactly as the reference's (which, built for x86-64, has no
fused multiply-add either).
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libso3g_gb300.so"
LIB = os.path.join(LIBDIR, LIBNAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xptxas", "-warn-spills"]
UNITS = ["api.cu", "pointing.cu", "scatter.cu", "scatter_weight.cu", "gather.cu", "precomp.cu",
         "noalloc.cu", "batch.cu", "batch_weight.cu", "sightline.cu", "ranges.cu"]
HEADERS = ["device.cuh", "host.h", "scatter_kernel.cuh", "scatter_launch.cuh", "batch_launch.cuh",
           "fastpoint.cuh", "mixedpoint.cuh", "mixed_launch.cuh", "mx_common.cuh", "interp_point.cuh"]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    """Compile and link the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "so3g_gb300.h")]
    jobs = []
    objs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs + [__file__]):
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-I", INCLUDE, "-c", src, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _stale(LIB, objs):
        # Link to a temporary name and rename, so a running process that has
        # the old library mapped is not disturbed.
        tmp = LIB + ".tmp"
        _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
