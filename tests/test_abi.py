"""CPU checks of the C ABI: the library loads and exports every entry point
declared in include/*.h; the host-only small-matrix routines work.  No GPU
calls are made here."""
import ctypes
import glob
import os
import re

import numpy as np

from blopex_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for path in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
        src = re.sub(r"typedef\s+struct\s*\{.*?\}\s*\w+\s*;", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", src, re.M | re.S):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    declared = declared_functions()
    assert len(declared) >= 70
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    assert declared <= set(_lib.SIGNATURES), declared - set(_lib.SIGNATURES)


def test_library_is_built_for_sm103a():
    # the build recipe targets exactly one architecture
    from blopex_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_fortran_matrix_host_routines():
    lib = _lib.load()
    m = lib.utilities_FortranMatrixCreate()
    lib.utilities_FortranMatrixAllocateData(4, 4, m)
    vals = ctypes.cast(lib.utilities_FortranMatrixValues(m), ctypes.POINTER(ctypes.c_double))
    rng = np.random.default_rng(0)
    u = np.triu(rng.uniform(1, 2, (4, 4)))
    for j in range(4):
        for i in range(4):
            vals[i + 4 * j] = u[i, j]
    lib.utilities_FortranMatrixUpperInv(m)
    inv = np.array([[vals[i + 4 * j] for j in range(4)] for i in range(4)])
    np.testing.assert_allclose(np.triu(inv) @ u, np.eye(4), atol=1e-14)
    assert lib.utilities_FortranMatrixGlobalHeight(m) == 4
    blk = lib.utilities_FortranMatrixCreate()
    lib.utilities_FortranMatrixSelectBlock(m, 2, 3, 2, 4, blk)
    assert lib.utilities_FortranMatrixHeight(blk) == 2 and lib.utilities_FortranMatrixWidth(blk) == 3
    lib.utilities_FortranMatrixDestroy(blk)
    lib.utilities_FortranMatrixDestroy(m)


def _header_struct(name):
    """[(field, C type)] of `typedef struct { ... } name;` in lobpcg_gb300.h."""
    src = open(os.path.join(ROOT, "include", "lobpcg_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef\s+struct\s*\{((?:(?!typedef).)*?)\}\s*" + name + r"\s*;", src,
                     re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m = re.match(r"(.*?)\s*\b(\w+)\s*(\[\s*\d+\s*\])?$", decl)
        out.append((m.group(2), m.group(1) + (m.group(3) or "")))
    return out


_CTYPES = {"int": ctypes.c_int, "double": ctypes.c_double, "long long": ctypes.c_longlong}


def test_python_structs_mirror_the_header():
    """The ctypes mirrors of the options and statistics structs have the
    header's fields, in order and with the same types (a mismatch would
    silently shift every later field)."""
    for cname, py in (("lobpcg_gpu_options", _lib.Options), ("lobpcg_gpu_stats", _lib.Stats)):
        fields = _header_struct(cname)
        assert [f for f, _ in fields] == [f for f, _ in py._fields_], cname
        for (f, ctype), (_, pytype) in zip(fields, py._fields_):
            assert _CTYPES[ctype] is pytype, (cname, f, ctype, pytype)
    kt = _header_struct("lobpcg_gpu_kernel_time")
    assert [f for f, _ in kt] == [f for f, _ in _lib.KernelTime._fields_]


def test_c_caller_compiles_and_links(tmp_path):
    """A C99 program calling lobpcg_solve_double the reference driver's way
    (tests/c/serial_driver_gb300.c) compiles warning-free against include/
    and links against the library: the headers are plain C and every symbol
    a C caller uses resolves.  (Running it needs the GPU.)"""
    import shutil
    import subprocess
    import pytest
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    libdir = os.path.dirname(_lib.LIBPATH)
    exe = tmp_path / "serial_driver_gb300"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "serial_driver_gb300.c"), "-L", libdir,
           "-llobpcg_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert exe.exists()
