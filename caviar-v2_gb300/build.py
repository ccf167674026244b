"""Build libcavgpu.so (the sm_103a kernels + the C ABI of include/cavgpu.h) in-tree.

Each .cu file compiles in parallel with nvcc for sm_103a only, then links into
caviar-v2_gb300/libcavgpu.so.  No CMake; runs in a few tens of seconds.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcavgpu.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
         "-diag-suppress", "1444"]
SOURCES = ["cav_kernels.cu", "cav_force.cu", "cav_api.cu", "cav_peaks.cu", "cav_noalloc.cu"]


def _compile(src, verbose):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [NVCC, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", out]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    return out, r.stderr


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    objs = [o for o, _ in results]
    cmd = [NVCC, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    build_host()
    return LIB


HOST_LIB = os.path.join(HERE, "libcaviar2_gpu.so")
LJ_MD = os.path.join(OBJ, "lj_md")


def build_host():
    """The CAVIAR2-shaped C++ API (host/) over libcavgpu.so and the lj_md driver."""
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(HERE, "host")]
    cxx = os.environ.get("CXX", "g++")
    steps = [
        [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-fPIC", "-shared", *inc,
         os.path.join(HERE, "host", "caviar2_gpu.cpp"), "-o", HOST_LIB, "-L" + HERE, "-lcavgpu", "-Wl,-rpath,$ORIGIN"],
        [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", *inc, os.path.join(HERE, "host", "lj_md.cpp"),
         "-o", LJ_MD, "-L" + HERE, "-lcaviar2_gpu", "-lcavgpu", "-Wl,-rpath," + HERE],
    ]
    for cmd in steps:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host build failed ({' '.join(cmd[:3])} ...):\n{r.stderr}")
    return HOST_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
