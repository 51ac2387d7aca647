"""The C-ABI library loads and exports exactly what include/sphx.h declares.

No compute call runs here (this suite also runs on machines without a GPU).
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import sphx

HEADER = Path(__file__).resolve().parents[1] / "include" / "sphx.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sphx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_binding_surface():
    assert declared_functions() == sorted(sphx.EXPORTS)


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(str(sphx.LIB_PATH))
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version_and_error_strings(built):
    lib = sphx.lib()
    assert lib.sphx_version() == 3
    for code in range(-8, 1):
        assert lib.sphx_strerror(code)


def test_struct_layouts_match_header():
    # 16 floats in SPHParameters order; fixed-width stats record
    assert C.sizeof(sphx.SphxParams) == 64
    assert [f for f, _ in sphx.SphxParams._fields_][-1] == "neighbor_search_radius"
    assert C.sizeof(sphx.SphxTuning) == 40  # 7 ints + int64
    assert C.sizeof(sphx.SphxStats) == 5 * 8 + 3 * 8 + 2 * 4 + 4 * 4 + 7 * 8 + 8 + 2 * 4


def test_null_context_arguments_are_rejected(built):
    lib = sphx.lib()
    assert lib.sphx_create(None, 10, None) == -1
    n = C.c_size_t()
    assert lib.sphx_size(None, C.byref(n)) == -1
    assert lib.sphx_step(None, C.c_float(0.0)) == -1


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(ImportError):
        sphx.load_library(tmp_path / "nope.so")
