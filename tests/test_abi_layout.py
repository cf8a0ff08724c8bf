"""The ctypes mirrors of the C ABI's structs (graspan-g_gb300/grg.py: Stats = grg_stats,
PartStats = grg_part_stats) against include/grg.h: a C program compiled here from the
Python field lists prints each field's offset and size and the struct sizes, which must
match ctypes' layout field for field. No GPU needed."""
import ctypes
import os
import shutil
import subprocess

import pytest

import grg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("cls, cname", [(grg.Stats, "grg_stats"), (grg.PartStats, "grg_part_stats")])
def test_struct_layout_matches_header(tmp_path, cls, cname):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "grg.h"', 'int main(void) {',
             f'    printf("sizeof %zu\\n", sizeof({cname}));']
    for name, _ in cls._fields_:
        lines.append(f'    printf("{name} %zu %zu\\n", offsetof({cname}, {name}), sizeof((({cname} *)0)->{name}));')
    lines += ['    return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                                check=True).stdout.splitlines())
    assert int(out.pop("sizeof")) == ctypes.sizeof(cls), cname
    for name, _ in cls._fields_:
        off, size = map(int, out[name].split())
        field = getattr(cls, name)
        assert (off, size) == (field.offset, field.size), (cname, name)
