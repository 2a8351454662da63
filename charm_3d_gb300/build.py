"""Build libcharm_gpu.so in-tree: CUDA kernels for sm_103a plus the host C code.

Used by ``__graft_entry__.build()`` and by the tests/bench when the library is
missing.  No cmake: nvcc and gcc are invoked directly, translation units in
parallel, one ``-gencode`` (compute_103a / sm_103a).
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
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libcharm_gpu.so")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_SOURCES = ["charm_gpu.cu", "charm_p2.cu", "charm_point.cu", "charm_tc.cu", "charm_dw.cu", "charm_hex.cu"]
C_SOURCES = ["host/charm_forest.c", "host/charm_host_api.c", "host/charm_yaml.c", "host/charm_case.c",
             "host/charm_conn.c"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcharm_gpu.so")


def _run(cmd: list[str]) -> str:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def _objects(verbose_ptxas: bool) -> list[tuple[list[str], str]]:
    nvcc = _nvcc()
    jobs = []
    inc = ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(CSRC, "host")]
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
               os.path.join(CSRC, src), "-o", obj] + inc
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
        jobs.append((cmd, obj))
    for src in C_SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-Wall", "-ffp-contract=off", "-pthread", "-c",
               os.path.join(CSRC, src), "-o", obj] + inc
        jobs.append((cmd, obj))
    return jobs


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile and link libcharm_gpu.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    sources = [os.path.join(CSRC, s) for s in CUDA_SOURCES + C_SOURCES]
    headers = [os.path.join(dp, f) for dp, _, fs in os.walk(CSRC) for f in fs if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "charm_gpu.h"))
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in sources + headers)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    jobs = _objects(verbose_ptxas)
    # recompile an object only when it is missing or older than its source
    # or any header (all translation units share the headers)
    newest_header = max(os.path.getmtime(p) for p in headers)
    todo = [j for j in jobs if force or verbose_ptxas or not os.path.exists(j[1]) or
            os.path.getmtime(j[1]) < max(newest_header, os.path.getmtime(j[0][j[0].index("-c") + 1]))]
    with cf.ThreadPoolExecutor(max_workers=max(1, len(todo))) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), todo))
    if verbose_ptxas:
        sys.stderr.write("".join(logs))
    objs = [o for _, o in jobs]
    tmp = LIB + ".tmp"
    _run([_nvcc(), GENCODE, "-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
