"""Build the sm_103a shared library ``peps_mg_gb300/lib/libpeps_mg.so`` in place.

Each translation unit is compiled by its own nvcc process (in parallel), then linked
with the static CUDA runtime.  FP64 translation units that must reproduce the
reference's non-FMA arithmetic get ``--fmad=false``; host code everywhere gets
``-ffp-contract=off`` (GCC on aarch64 would otherwise fuse a*b+c).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIBDIR, "libpeps_mg.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3"]

# translation unit -> extra flags
UNITS = {
    "pmg_api.cu": ["--fmad=false"],
    "pmg_f64.cu": ["--fmad=false"],
    "pmg_f64fast.cu": ["--fmad=true"],
    "pmg_mixed.cu": ["--fmad=true"],
    "pmg_smooth32.cu": ["--fmad=true"],
    "pmg_batch.cu": ["--fmad=true"],
    "pmg_adjoint.cu": ["--fmad=false"],
    "pmg_dot_static.cu": ["--fmad=false"],
    "pmg_dd.cu": ["--fmad=false"],
}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build peps_mg_gb300")
    return path


def _headers_mtime():
    t = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(unit, flags, force):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJDIR, unit.replace(".cu", ".o"))
    if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and os.path.getmtime(obj) >= _headers_mtime()):
        return obj, ""
    cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), p.stderr))
    return obj, p.stderr


def build(force=False, verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, u, f, force) for u, f in UNITS.items()]
        objs = []
        for fu in futs:
            obj, log = fu.result()
            objs.append(obj)
            if verbose and log:
                print(log, file=sys.stderr)
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), p.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
