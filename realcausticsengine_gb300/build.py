"""Build librealcaustics.so in-tree (nvcc for sm_103a, g++ for pure host files).

Every translation unit is compiled without floating-point contraction
(-fmad=false on the device, -ffp-contract=off on the host): the closest-hit,
BVH-build and KD-query paths rely on each float operation rounding as written.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "librealcaustics.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", f"-I{ROOT / 'include'}", f"-I{CSRC}"]
GXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{ROOT / 'include'}", f"-I{CSRC}"]

# (source, compiler): .cu and device-header users through nvcc, pure host C++ through g++
SOURCES = [
    ("host_scene.cpp", "gxx"),
    ("rc_abi.cpp", "nvcc"),
    ("vm_kernels.cu", "nvcc"),
    ("gather.cu", "nvcc"),
    ("kdtree.cu", "nvcc"),
    ("kd_noalloc.cu", "nvcc"),
    ("vm_mlt.cu", "nvcc"),
    ("tc_selftest.cu", "nvcc"),
    ("mlp.cu", "nvcc"),
    ("bvh_build.cu", "nvcc"),
]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, kind: str, extra: list[str]) -> Path:
    out = BUILD / (Path(src).stem + ".o")
    s = CSRC / src
    if kind == "nvcc":
        cmd = [_nvcc(), *NVCC_FLAGS, *extra, "-x", "cu", "-c", str(s), "-o", str(out)]
    else:
        cmd = ["g++", *GXX_FLAGS, "-I/usr/local/cuda/include", "-c", str(s), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda sk: _compile(sk[0], sk[1], extra), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
