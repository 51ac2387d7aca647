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


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every ctypes mirror has the C struct's size and each field's C offset: a small C
    program compiled against include/sphx.h prints them (a field missing from the header
    fails the compile)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [(sphx.SphxParams, "sphx_params"), (sphx.SphxTuning, "sphx_tuning"),
             (sphx.SphxStats, "sphx_stats"), (sphx.SphxSceneStats, "sphx_scene_stats"),
             (sphx.SphxShape, "sphx_shape"), (sphx.SphxRenderParams, "sphx_render_params")]
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "sphx.h"', "int main(void) {"]
    expect = []
    for cls, cname in pairs:
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append(C.sizeof(cls))
        for field, _ in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {field}));')
            expect.append(getattr(cls, field).offset)
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", f"-I{HEADER.parent}", str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == expect
