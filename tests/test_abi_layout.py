"""The ctypes mirrors of the C-ABI structs (heomq) against the header itself: a small C
program built with the host compiler prints every field's offset and every struct's size,
and the Python structures must match them field by field (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

import heomq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "heom_tables": heomq.Tables,
    "heom_params": heomq.Params,
    "heom_ctx_opts": heomq.CtxOpts,
    "heom_solve_opts": heomq.SolveOpts,
    "heom_solve_info": heomq.SolveInfo,
    "heom_cf_tables": heomq.CfTables,
    "heom_grad_opts": heomq.GradOpts,
}


@pytest.fixture(scope="module")
def layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no host C compiler")
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "heom_gb300.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        src.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            src.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    src += ["return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    c = d / "layout.c"
    c.write_text("\n".join(src))
    exe = d / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        s, f, v = line.split()
        table[(s, f)] = int(v)
    return table


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_struct_matches_the_header(layout, cname):
    py = STRUCTS[cname]
    import ctypes

    assert ctypes.sizeof(py) == layout[(cname, "size")], cname
    for fname, _ in py._fields_:
        assert getattr(py, fname).offset == layout[(cname, fname)], (cname, fname)
