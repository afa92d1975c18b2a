"""CPU-side checks of the C-ABI library: it builds for sm_103a, loads, and
exports every entry point that include/si_gpu/c_api.h declares (no GPU call)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "si_gpu", "c_api.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:[A-Za-z_][A-Za-z0-9_]*\s+)*[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**"
                       r"([A-Za-z_][A-Za-z0-9_]*)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from superintervals_gb300 import build_ext, _capi
    build_ext.build()
    return _capi.load()


def test_header_declares_the_path_entry_points():
    names = declared_functions()
    for must in ("createSuperIntervalsGpu", "indexSuperIntervalsGpu", "countOverlapsBatchGpu",
                 "searchIdxsBatchGpu", "searchValuesBatchGpu", "anyOverlapsBatchGpu",
                 "searchDeviceGpu", "destroyCsrResult"):
        assert must in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(lib):
    from superintervals_gb300 import _capi
    assert set(declared_functions()) == set(_capi.SIGNATURES)


def test_library_is_built_for_sm_103a_only():
    from superintervals_gb300 import build_ext
    assert build_ext.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_product_package_does_not_touch_the_oracle():
    pkg = os.path.join(ROOT, "superintervals_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".hpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in text.replace("the oracle is the oracle", ""), f
