"""In-tree build of the native libraries (no cmake, no pip install).

* ``_build/libchanga_gb300.so`` -- the CUDA library (sm_103a kernels and the
  C-ABI of include/HostCUDA.h, include/EwaldCUDA.h, include/changa_gb300.h).
* ``_build/libchanga_gb300_hex.so`` -- the same library built with
  -DHEXADECAPOLE: the boundary of ChaNGa's hexadecapole build.
* ``_build/libchanga_host.so`` -- host tree build, dual walk and list
  serialisation (the caller side of the boundary).

Translation units compile in parallel; nvcc targets sm_103a only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["grav_lists.cu", "ewald.cu", "hostcuda.cu", "noalloc.cu", "adjoint.cu",
              "moments.cu", "direct.cu", "walk.cu",
              "treebuild.cu"]
CXX_SOURCES = ["cxx_abi.cpp", "ewald_table.cpp"]
# Sources whose FP64 results must equal the host code's bit for bit: no FMA
# contraction, as the host library is compiled with -ffp-contract=off.
NO_FMA_SOURCES = {"treebuild.cu": ["-fmad=false"], "walk.cu": ["-fmad=false"]}

CUDA_LIB = os.path.join(BUILD, "libchanga_gb300.so")
# the same sources with -DHEXADECAPOLE: the boundary of ChaNGa's default
# (hexadecapole) build, 108-byte CudaMultipoleMoments and the hexadecapole
# Ewald root expansion
HEX_LIB = os.path.join(BUILD, "libchanga_gb300_hex.so")
HOST_LIB = os.path.join(BUILD, "libchanga_host.so")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _openmp_flag():
    probe = os.path.join(BUILD, "_omp_probe.c")
    with open(probe, "w") as f:
        f.write("#include <omp.h>\nint main(void){return omp_get_max_threads() > 0 ? 0 : 1;}\n")
    r = subprocess.run(["gcc", "-fopenmp", probe, "-o", probe + ".bin"],
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    for p in (probe, probe + ".bin"):
        if os.path.exists(p):
            os.remove(p)
    return ["-fopenmp"] if r.returncode == 0 else []


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def build_host(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(PKG, "host", "tree.cpp")
    if not force and _newer(HOST_LIB, [src]):
        return HOST_LIB
    cmd = ["g++", "-O3", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off"] + _openmp_flag() + \
          [src, "-o", HOST_LIB]
    _run(cmd)
    return HOST_LIB


def build_cuda(force=False, verbose=False):
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    headers = [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE)] + \
              [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CXX_SOURCES]
    if not force and _newer(CUDA_LIB, srcs + headers) and _newer(HEX_LIB, srcs + headers):
        return CUDA_LIB
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at %s" % NVCC)
    inc = ["-I" + INCLUDE, "-I" + CSRC]
    jobs = []
    objs = {CUDA_LIB: [], HEX_LIB: []}
    for lib, odir, defs in ((CUDA_LIB, "obj", []), (HEX_LIB, "obj_hex", ["-DHEXADECAPOLE"])):
        os.makedirs(os.path.join(BUILD, odir), exist_ok=True)
        for s in CU_SOURCES:
            o = os.path.join(BUILD, odir, s + ".o")
            objs[lib].append(o)
            extra = NO_FMA_SOURCES.get(s, [])
            jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-Xptxas", "-v"] + extra + defs + inc +
                        ["-c", os.path.join(CSRC, s), "-o", o])
        for s in CXX_SOURCES:
            o = os.path.join(BUILD, odir, s + ".o")
            objs[lib].append(o)
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off",
                         "-I" + os.path.join(CUDA_HOME, "include")] + defs + inc +
                        ["-c", os.path.join(CSRC, s), "-o", o])
    with ThreadPoolExecutor(max_workers=min(len(jobs), (os.cpu_count() or 8) * 2)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    # -Bsymbolic: each library binds its own internal references, so the two
    # builds (same symbol names) can share one process
    for lib in (CUDA_LIB, HEX_LIB):
        _run([NVCC] + ARCH + ["-shared", "-Xlinker", "-Bsymbolic", "-o", lib] + objs[lib])
    with open(os.path.join(BUILD, "ptxas.txt"), "w") as f:
        f.write("".join(outs))
    return CUDA_LIB


def build_oracle():
    """Builds oracle/ (the CPU checker) with its own Makefile."""
    odir = os.path.join(ROOT, "oracle")
    if not os.path.isdir(odir) or shutil.which("make") is None:
        return False
    _run(["make", "-s", "-C", odir])
    return True


def build_all(force=False, verbose=False):
    build_host(force)
    build_cuda(force, verbose)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    build_oracle()
    print("built", CUDA_LIB, HOST_LIB)
