"""The ctypes mirrors of the C ABI's structs (sqminiapp_gb300/capi.py) against the header:
gcc compiles a probe that prints sizeof and every member's offsetof, and each must equal the
ctypes layout (a field added on one side only would shift every later field)."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _probe(tmp_path, structs):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sq_gb300.h"', 'int main(void) {']
    for cname, fields in structs.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in fields:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        out[(s, f)] = int(v)
    return out


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_the_header(tmp_path):
    from sqminiapp_gb300.capi import (SqInfo, SqOptions, SqPsdDesc, SqScfOptions, SqScfResult,
                                      SqSystemDesc)
    mirrors = {"sq_options": SqOptions, "sq_info": SqInfo, "sq_scf_options": SqScfOptions,
               "sq_scf_result": SqScfResult, "sq_psd_desc": SqPsdDesc,
               "sq_system_desc": SqSystemDesc}
    c = _probe(tmp_path, {n: [f for f, _ in m._fields_] for n, m in mirrors.items()})
    for n, m in mirrors.items():
        assert c[(n, "sizeof")] == ctypes.sizeof(m), n
        for f, _ in m._fields_:
            assert c[(n, f)] == getattr(m, f).offset, (n, f)
