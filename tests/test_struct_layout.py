"""The ctypes mirrors of the C ABI's structs (isar_imaging_cuda_gb300) agree
with include/isar_gb300.h: same field names, offsets and sizes, checked with
a small C program compiled by gcc against the header (CPU only)."""
import ctypes as C
import json
import os
import shutil
import subprocess

import pytest

import isar_imaging_cuda_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TMP = os.path.join(ROOT, "tests", "_tmp", "layout")

STRUCTS = {"isar_radar": g.Radar, "isar_trace": g.Trace, "isar_tuning": g.Tuning,
           "isar_synth_params": g.SynthParams, "isar_batch_frame": g.BatchFrame}


def c_layout():
    os.makedirs(TMP, exist_ok=True)
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "isar_gb300.h"', 'int main(void) {',
             '  printf("{");']
    first = True
    for cname, py in STRUCTS.items():
        sep = "" if first else ","
        first = False
        lines.append('  printf("%s\\"%s\\": {\\"size\\": %%zu", sizeof(%s));' % (sep, cname, cname))
        for f, _ in py._fields_:
            lines.append('  printf(", \\"%s\\": %%zu", offsetof(%s, %s));' % (f, cname, f))
        lines.append('  printf("}");')
    lines += ['  printf("}\\n");', '  return 0;', '}']
    src = os.path.join(TMP, "layout.c")
    exe = os.path.join(TMP, "layout")
    open(src, "w").write("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
    return json.loads(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_structs_match_the_header():
    lay = c_layout()
    for cname, py in STRUCTS.items():
        got = lay[cname]
        assert got["size"] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[f] == getattr(py, f).offset, (cname, f)
