"""Build libgbfem.so (CUDA, sm_103a) and the CPU oracle.

nvcc compiles each translation unit in parallel into _build/, then links
femx_gb300/libgbfem.so with a static CUDA runtime. Only one -gencode is
used: the library targets GB300 (sm_103a) and nothing else.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libgbfem.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["core.cu", "pattern.cu", "boundary.cu", "p1.cu", "spmv.cu", "th.cu", "measure.cu",
           "noalloc.cu", "batch.cu", "transpose.cu", "tiles.cu",
           "navier.cu", "gmsh.cu", "hostio.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libgbfem")
    return cand


def _newest_dep() -> float:
    files = [f for f in glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "*.h"))
             if not f.endswith("pycore.cpp")]
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def _core_path() -> str:
    return os.path.join(PKG, "_core" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_core(force: bool = False) -> str:
    """Build the pybind11 module femx_gb300._core (femx's Python surface for
    the assembly path) against libgbfem.so, with the pybind11 headers that
    ship with torch and the interpreter's headers. Host C++ only (g++)."""
    lib = build()
    out = _core_path()
    src = os.path.join(CSRC, "pycore.cpp")
    deps = [lib, src, os.path.join(INCLUDE, "gbfem.h")]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(f) for f in deps):
        return out
    import torch.utils.cpp_extension as ext
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("g++ not found: needed to build femx_gb300._core")
    incs = [sysconfig.get_paths()["include"], INCLUDE] + ext.include_paths()[:1]
    tmp = out + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
           *["-I" + i for i in incs], src, "-L" + PKG, "-l:libgbfem.so",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"femx_gb300._core build failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, out)
    return out


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_dep():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
    print(build_core(force=True))
