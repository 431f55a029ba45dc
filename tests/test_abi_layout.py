"""The ctypes mirrors of the C-ABI structs have the C layout: for every public struct declared in
include/*.h that the Python host binds, sizeof and the offset of every member agree with what a C
compiler makes of the header (gcc on the headers alone; no library or device involved)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from multiq_workbench_gb300 import _native as N

ROOT = Path(__file__).resolve().parents[1]
HEADERS = ("mq_engine.h", "mq_grid.h", "mq_tandem.h", "mq_fit.h")


def _structs():
    out = []
    for name in dir(N):
        obj = getattr(N, name)
        if isinstance(obj, type) and issubclass(obj, C.Structure) and obj is not C.Structure and name.startswith("mq_"):
            out.append(obj)
    return sorted(out, key=lambda s: s.__name__)


def test_every_bound_struct_is_checked():
    names = {s.__name__ for s in _structs()}
    assert {"mq_job", "mq_physics", "mq_outcome", "mq_ions", "mq_run_stats", "mq_tuning", "mq_grid_desc",
            "mq_tandem_desc", "mq_res_fit"} <= names


def test_struct_layouts_match_the_headers(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>"] + [f'#include "{h}"' for h in HEADERS]
    lines.append("int main(void) {")
    for s in _structs():
        n = s.__name__
        lines.append(f'    printf("{n} sizeof %zu\\n", sizeof({n}));')
        for fname, _ in s._fields_:
            lines.append(f'    printf("{n} {fname} %zu\\n", offsetof({n}, {fname}));')
    lines.append("    return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        struct, member, value = line.split()
        got[(struct, member)] = int(value)
    bad = []
    for s in _structs():
        n = s.__name__
        if got[(n, "sizeof")] != C.sizeof(s):
            bad.append(f"{n}: sizeof C {got[(n, 'sizeof')]} vs ctypes {C.sizeof(s)}")
        for fname, _ in s._fields_:
            off = getattr(s, fname).offset
            if got[(n, fname)] != off:
                bad.append(f"{n}.{fname}: offset C {got[(n, fname)]} vs ctypes {off}")
    assert not bad, "\n".join(bad)
