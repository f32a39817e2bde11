"""Builds libint_gb300/liblgx.so (CUDA kernels + C ABI + host utilities).

Every CUDA translation unit is compiled for sm_103a only; translation units
compile in parallel and link into one in-tree shared library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(PKG_DIR, "liblgx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["lgx_kernels.cu", "lgx_api.cu", "lgx_boys.cu"]
CXX_SOURCES = ["lgx_program.cpp", "lgx_host.cpp", "lgx_libint_c.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblgx")


def _generate() -> list:
    """Regenerates the unrolled per-class code (files are rewritten only when
    their content changes); returns the generated CUDA units (csrc/gen)."""
    sys.path.insert(0, os.path.join(PKG_DIR, "codegen"))
    try:
        import gen_rk
        import gen_post
        units = gen_rk.main() + gen_post.main()
    finally:
        sys.path.pop(0)
    return [os.path.join("gen", u) for u in units]


def _deps_mtime() -> float:
    t = 0.0
    for d in (CSRC, os.path.join(CSRC, "gen"), os.path.join(PKG_DIR, "codegen"),
              os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            fp = os.path.join(d, f)
            if os.path.isfile(fp):
                t = max(t, os.path.getmtime(fp))
    return t


def build(force: bool = False, verbose: bool = False) -> str:
    cuda_sources = CUDA_SOURCES + _generate()
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= _deps_mtime()):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for src in cuda_sources:
        obj = os.path.join(BUILD_DIR, src.replace("/", "_") + ".o")
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17",
                     "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                     "-c", os.path.join(CSRC, src), "-o", obj])
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD_DIR, src + ".o")
        jobs.append(["g++", "-std=c++17", "-O3", "-fPIC", "-c",
                     os.path.join(CSRC, src), "-o", obj])

    # skip objects newer than their source and every header
    hdr = 0.0
    for d in (CSRC, os.path.join(CSRC, "gen"), os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                hdr = max(hdr, os.path.getmtime(os.path.join(d, f)))
    if not force:
        jobs = [j for j in jobs if not (os.path.exists(j[-1]) and os.path.getmtime(j[-1]) >=
                                        max(hdr, os.path.getmtime(j[-3])))]

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stdout + r.stderr

    # biggest units first so the parallel build ends evenly
    jobs.sort(key=lambda j: -os.path.getsize(j[-3]))
    workers = max(2, min(max(len(jobs), 1), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=workers) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        print("".join(logs))
    objs = [os.path.join(BUILD_DIR, s.replace("/", "_") + ".o") for s in cuda_sources + CXX_SOURCES]
    tmp = LIB_PATH + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
