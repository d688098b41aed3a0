"""The C-ABI library builds, loads and exports every symbol include/sstmc.h declares."""
import ctypes as C
import os
import re

import pytest

from temporalspecklescode_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sstmc.h")).read()
    return sorted(set(re.findall(r"\b(sstmc_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_build.lib_path()):
        _build.build_library()
    return C.CDLL(_build.lib_path())


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert "sstmc_render" in syms and "sstmc_scene_create" in syms
    for s in syms:
        assert hasattr(lib, s), s


def test_error_strings(lib):
    lib.sstmc_error_string.restype = C.c_char_p
    assert lib.sstmc_error_string(0) == b"No error."
    assert b"Allocation" in lib.sstmc_error_string(2)
    assert b"not supported" in lib.sstmc_error_string(5)
    assert lib.sstmc_error_string(999) == b"Unknown error code."


def test_null_handles_are_rejected(lib):
    assert lib.sstmc_render(None, C.c_uint64(0), None, None) == 103
    assert lib.sstmc_scene_destroy(None) == 103
