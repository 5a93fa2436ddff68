"""The Python binding's ctypes structures against the C header: every struct of
include/heterogpc.h has the same size and field offsets in both (a C program compiled
with the host compiler prints them). Guards the ABI whenever a struct or HPC_MAX_LEVEL
changes."""
import os
import shutil
import subprocess
import tempfile

import pytest

import heterogpc as hg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "hpc_opts": hg.Opts,
    "hpc_level_stats": hg.LevelStats,
    "hpc_sepset_record": hg.SepsetRecord,
    "hpc_timings": hg.Timings,
    "hpc_server_opts": hg.ServerOpts,
    "hpc_served": hg.Served,
    "hpc_sem_params": hg.SemParams,
    "hpc_tune_params": hg.TuneParams,
}


def test_struct_layouts_match_the_header():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "heterogpc.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True,
                       capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            a, b, v = ln.split()
            got[(a, b)] = int(v)
    for cname, py in STRUCTS.items():
        assert got[(cname, "size")] == __import__("ctypes").sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_max_level_constant_matches():
    hdr = open(os.path.join(ROOT, "include", "heterogpc.h")).read()
    assert "#define HPC_MAX_LEVEL %d" % hg.HPC_MAX_LEVEL in hdr
