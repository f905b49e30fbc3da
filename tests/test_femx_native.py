"""gbfem's femx-native adapter (include/gbfem/femx_native.cuh) compiled and
linked against femx's own headers and femx's own library, the way a femx
user builds it: femx's Mesh / makeGeometry / makeAssemblyMap produce the
inputs; the adapter's Residual<CudaCsrBackend> and TimeResidual<CudaCsrBackend>
subclasses go to code written against femx's interfaces only; femx's
assemble signature over femx's device types resolves and links
(tests/cpp/femx_native_test.cu).

Needs the femx source tree ($FEMX_REFERENCE, or `reference` beside this
repository) and its host library built by oracle/ref/Makefile; skipped where
either is absent (the GPU machine has neither). Without a CUDA device the program
stops after the host-side steps.
"""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "femx_native_test.cu")
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libfemx_ref.a")


def _reference():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g
    return g.reference_tree()


def test_adapter_builds_against_femx_and_runs_its_host_side(tmp_path):
    ref = _reference()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if ref is None or not os.path.exists(REFLIB) or not os.path.exists(nvcc):
        pytest.skip("femx source tree, its host library or nvcc not available")
    from femx_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "femx_native_test")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O1",
           "-diag-suppress", "20012", "-I" + ref, "-I" + os.path.join(ROOT, "include"), SRC,
           REFLIB, "-L" + os.path.dirname(lib), "-lgbfem",
           "-Xlinker", "-rpath," + os.path.dirname(lib), "-Xcompiler", "-fopenmp", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    p = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "host: 25 nodes, 32 elements, P1 nnz 137" in p.stdout
    assert "SKIP" in p.stdout or "device passes done" in p.stdout
