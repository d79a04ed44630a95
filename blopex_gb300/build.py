"""Build recipe for liblobpcg_gb300.so (sm_103a only, in-tree).

    python -m blopex_gb300.build          # or __graft_entry__.build()

Each translation unit is compiled in parallel (nvcc for the CUDA files, the
host C compiler for the C files) and linked with the static CUDA runtime
into ``blopex_gb300/_lib/liblobpcg_gb300.so``.  No cmake, no torch build
machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIBNAME = "liblobpcg_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(CSRC) if f.endswith(".c"))
    return cu, c


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cc = os.environ.get("CC", "gcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu, c = sources()
    jobs = []
    objs = []
    for f in cu:
        obj = os.path.join(BUILD, f + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, f), "-o", obj]
        if ptxas_info:
            cmd[1:1] = ["-Xptxas", "-v"]
        jobs.append(cmd)
        objs.append(obj)
    for f in c:
        obj = os.path.join(BUILD, f + ".o")
        cmd = [cc, "-O2", "-fPIC", "-std=c11", "-Wall", "-Wno-unused-function",
               "-I", INCLUDE, "-I", CSRC, "-I", os.path.join(cuda, "include"),
               "-c", os.path.join(CSRC, f), "-o", obj]
        jobs.append(cmd)
        objs.append(obj)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    lib = os.path.join(LIBDIR, LIBNAME)
    tmp = lib + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-Xlinker", "-Bsymbolic",
          "-o", tmp, *objs])
    os.replace(tmp, lib)
    if verbose or ptxas_info:
        sys.stderr.write("".join(logs))
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
