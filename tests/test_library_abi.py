"""CPU-side checks of the C ABI: the library builds, loads without a GPU and
exports every function include/gbfem.h declares; the ctypes signatures cover
the same set."""
import os
import re

import pytest

from femx_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(gbfem_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.lib()


def test_header_declares_the_path():
    names = declared_functions()
    for required in ("gbfem_assembly_map_create", "gbfem_boundary_map_create",
                     "gbfem_prepare_forward_solve", "gbfem_spmv", "gbfem_assemble_p1_kappa",
                     "gbfem_vjp_p1_kappa", "gbfem_assemble_th_ns"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_match_header():
    assert set(_lib.SIGNATURES) == set(declared_functions())


def test_version_and_error_plumbing_without_gpu(lib):
    assert lib.gbfem_version() >= 1
    # a null output handle is rejected on the host before any device work
    rc = lib.gbfem_assembly_map_create(1, 1, 0, None, None, None, None, None, None)
    assert rc == _lib.GBFEM_EINVAL
    assert "null" in lib.gbfem_last_error().decode()


def test_internal_symbols_are_hidden(lib):
    with pytest.raises(AttributeError):
        getattr(lib, "_ZN5gbfem12setLastErrorERKNSt7__cxx1112basic_stringIcSt11char_traitsIcESaIcEEE")
