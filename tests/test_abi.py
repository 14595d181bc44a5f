"""The C ABI library loads and exports every entry point include/gqf.h
declares (CPU only: no compute calls)."""
import ctypes
import os
import shutil
import subprocess

import pytest

import cqf_gb300
from cqf_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib_path():
    return gbuild.build()


def test_header_lists_the_reference_entry_points():
    names = cqf_gb300.exported_symbols_from_header(os.path.join(ROOT, "include", "gqf.h"))
    for ref in ("qf_malloc_device", "qf_destroy_device", "bulk_insert", "bulk_insert_reduce",
                "bulk_delete", "bulk_get", "bulk_get_misses_wrapper", "point_get_wrapper"):
        assert ref in names


def test_every_declared_symbol_is_exported(lib_path):
    lib = ctypes.CDLL(lib_path)
    names = cqf_gb300.exported_symbols_from_header(os.path.join(ROOT, "include", "gqf.h"))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python mirror binds exactly the declared set
    assert sorted(cqf_gb300.SIGNATURES) == names


def test_python_binding_loads(lib_path):
    L = cqf_gb300.load()
    assert L.gqf_version().decode().startswith("gqf_gb300")
    assert L.gqf_last_error().decode() == ""


@pytest.mark.skipif(shutil.which("nm") is None, reason="needs nm")
def test_device_library_defines_the_point_api(lib_path):
    out = subprocess.run(["nm", "-C", gbuild.DEVLIB_PATH], capture_output=True, text=True).stdout
    for sym in ("point_insert", "point_insert_not_exists", "point_query", "point_query_concurrent",
                "point_bulk_insert"):
        assert sym in out, sym
