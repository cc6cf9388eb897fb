"""The ctypes mirrors of the C ABI's structs match include/gbv.h field for
field: a small C program compiled here prints sizeof and offsetof of every
field, compared with the ctypes offsets (no GPU needed)."""
import ctypes
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

STRUCTS = {
    "gbv_cell_options": "CellOptions",
    "gbv_cell_report": "CellReport",
    "gbv_ot_options": "OtOptions",
    "gbv_ot_report": "OtReport",
    "gbv_mesh_sizes": "MeshSizes",
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from geogram_gb300 import _lib
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbv.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(_lib, pyname)
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        s, f, v = line.split()
        table[(s, f)] = int(v)
    return table


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_struct_layout(c_layout, cname):
    from geogram_gb300 import _lib
    cls = getattr(_lib, STRUCTS[cname])
    assert ctypes.sizeof(cls) == c_layout[(cname, "sizeof")]
    for f, _ in cls._fields_:
        assert getattr(cls, f).offset == c_layout[(cname, f)], f
