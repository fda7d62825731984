"""The C-ABI library: it loads without a GPU, exports exactly the entry
points include/vacgpu.h declares, and the ctypes mirror of vacgpu_params has
the C layout."""
import ctypes as C
import os
import re
import subprocess

import pytest

from vac_gb300 import abi, engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "vacgpu.h")


def declared_functions():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"^\w[\w\s\*]*?\b(vacgpu_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def built():
    from vac_gb300 import build
    build.build()
    return engine.lib()


def test_library_exports_every_declared_symbol(built):
    decl = declared_functions()
    assert len(decl) >= 12
    for name in decl:
        assert hasattr(built, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", engine.LIB],
                         capture_output=True, text=True).stdout
    exported = sorted(set(re.findall(r" T (vacgpu_\w+)", out)))
    assert exported == decl


def test_params_layout_matches_c(tmp_path, built):
    fields = [f[0] for f in abi.VacParams._fields_]
    src = tmp_path / "lay.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "%s"\n'
                   'int main(void){printf("%%zu\\n", sizeof(vacgpu_params));\n%s return 0;}\n'
                   % (HDR, "".join('printf("%%zu\\n", offsetof(vacgpu_params, %s));\n' % f
                                   for f in fields)))
    exe = tmp_path / "lay"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True,
                                           text=True).stdout.split()]
    assert vals[0] == C.sizeof(abi.VacParams)
    for f, off in zip(fields, vals[1:]):
        assert getattr(abi.VacParams, f).offset == off, f


def test_default_params_match_python_defaults(built):
    p = abi.VacParams()
    nx = (C.c_int * 3)(16, 8, 1)
    built.vacgpu_default_params(C.byref(p), 2, 2, abi.PHYS_MHD, nx)
    q = abi.default_params(2, 2, abi.PHYS_MHD, [16, 8])
    assert bytes(p) == bytes(q)


def test_create_rejects_bad_parameters_without_gpu(built):
    p = abi.default_params(2, 2, abi.PHYS_MHD, [16, 8])
    p.dixB = 3
    h = C.c_void_p()
    assert built.vacgpu_create(C.byref(p), C.byref(h)) != 0
    assert "dixB" in engine.last_error()
    p = abi.default_params(2, 2, abi.PHYS_MHD, [16, 8])
    p.typeB[0][0] = abi.BC_PERIODIC  # lower periodic without its pair
    assert built.vacgpu_create(C.byref(p), C.byref(h)) != 0
    assert "periodic pair" in engine.last_error()
