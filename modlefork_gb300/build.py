"""Build the GB300 epoch engine (libmgpu_modle.so) in-tree with nvcc for sm_103a.

The library holds the CUDA kernels and the C ABI (include/mgpu_modle.h).  Every double
multiply and add is rounded separately (--fmad=false on the device, -ffp-contract=off on the
host), the arithmetic contract the engine shares with the reference's x86-64 build.
"""

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libmgpu_modle.so")
SOURCES = ["mgpu_device.cu", "mgpu_pixels.cu", "mgpu_host.cpp"]
HEADERS = ["mgpu_internal.h", "cppsort_emul.h", "ziggurat_tables.h",
           os.path.join("..", "..", "include", "mgpu_modle.h")]
# The surrogate's kernels (tcgen05 / TMA convolutions and their companions): a library of its
# own, built without the engine's exact-rounding flags, which its FP32 arithmetic does not need.
SUR_LIB = os.path.join(LIBDIR, "libmgpu_surrogate.so")
SUR_SOURCES = ["surrogate.cu"]
SUR_HEADERS = ["umma.cuh", os.path.join("..", "..", "include", "mgpu_surrogate.h")]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")
    return path


def _stale(lib, sources, headers):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in sources + headers]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _start(lib, sources, common, verbose):
    """Start the compiles of one library; returns (lib, objs, procs)."""
    objs, procs = [], []
    for src in sources:
        obj = os.path.join(LIBDIR, src + ".o")
        cmd = [nvcc(), *common, "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd.insert(1, "-Xptxas=-v" if verbose else "-Xptxas=-O3")
        objs.append(obj)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    return lib, objs, procs


def _finish(lib, objs, procs, verbose, extra_link=()):
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + out.decode())
        if verbose and out:
            sys.stdout.write(out.decode())
    tmp = lib + ".tmp"
    link = [nvcc(), ARCH, "-shared", "-o", tmp, *objs, *extra_link]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode())
    os.replace(tmp, lib)
    for o in objs:
        os.remove(o)


def build(force=False, verbose=False):
    """Compile both libraries' translation units in parallel and link them."""
    os.makedirs(LIBDIR, exist_ok=True)
    inc = ["-I", os.path.join(PKG, "..", "include")]
    jobs = []
    if force or _stale(LIB, SOURCES, HEADERS):
        common = [ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
                  "-Xcompiler", "-fPIC,-ffp-contract=off", *inc]
        jobs.append(_start(LIB, SOURCES, common, verbose))
    if force or _stale(SUR_LIB, SUR_SOURCES, SUR_HEADERS):
        common = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *inc]
        jobs.append(_start(SUR_LIB, SUR_SOURCES, common, verbose))
    for lib, objs, procs in jobs:
        _finish(lib, objs, procs, verbose)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
