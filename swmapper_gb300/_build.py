"""Build recipes for the in-tree native libraries of the package.

Everything is compiled in place (no pip install): the CUDA library for sm_103a
with nvcc, the C host pieces and command-line tools with gcc.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")

LIB_CUDA = os.path.join(PKG, "libswmapper_gb300.so")
LIB_SYNTH = os.path.join(PKG, "libswm_synth.so")
BIN_INDEX = os.path.join(PKG, "swm_index")
BIN_MAP = os.path.join(PKG, "swm_mapper")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["swm_index.cu", "swm_map.cu", "swm_probe.cu", "swm_serve.cu"]
HOST_SOURCES = ["swm_files.c", "swm_sam.c"]


def _run(cmd: list[str], cwd: str | None = None) -> None:
    proc = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(proc.stdout + proc.stderr)
        raise RuntimeError("build step failed: " + " ".join(cmd))


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_synth() -> str:
    src = os.path.join(CSRC, "synth.c")
    deps = [src, os.path.join(INCLUDE, "swm_synth.h")]
    if not _newer(LIB_SYNTH, deps):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-I", INCLUDE, src, "-o", LIB_SYNTH])
    return LIB_SYNTH


def build_cuda() -> str:
    nvcc = _nvcc()
    objdir = os.path.join(PKG, "_build")
    os.makedirs(objdir, exist_ok=True)
    headers = [os.path.join(INCLUDE, "swmapper.h"), os.path.join(INCLUDE, "swm_sam.h"),
               os.path.join(CSRC, "swm_common.cuh")]
    objs = []
    jobs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(objdir, s + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(objdir, s + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + headers):
            jobs.append(["gcc", "-O2", "-fPIC", "-std=gnu11", "-I", INCLUDE, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if not _newer(LIB_CUDA, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB_CUDA, *objs, "-lcudart", "-lpthread"])
    return LIB_CUDA


def _have_zlib() -> bool:
    """zlib headers and library present (the mapper CLI then writes .sam.gz)."""
    probe = subprocess.run(["gcc", "-x", "c", "-", "-lz", "-o", os.devnull],
                           input="#include <zlib.h>\nint main(void){return zlibVersion()==0;}\n",
                           capture_output=True, text=True)
    return probe.returncode == 0


def build_cli() -> None:
    """swm_index and swm_mapper, the drop-ins for serial_index and the mapper."""
    zl = _have_zlib()
    for name, out in (("cli_index.c", BIN_INDEX), ("cli_mapper.c", BIN_MAP)):
        src = os.path.join(CSRC, name)
        if not os.path.exists(src):
            continue
        if not _newer(out, [src, LIB_CUDA, os.path.join(INCLUDE, "swmapper.h"), os.path.join(INCLUDE, "swm_sam.h")]):
            extra = ["-DHAVE_ZLIB"] if (zl and name == "cli_mapper.c") else []
            libs = ["-lz"] if extra else []
            _run(["gcc", "-O2", "-std=gnu11", *extra, "-I", INCLUDE, src, "-o", out,
                  "-L", PKG, "-lswmapper_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread", *libs])


def build_all() -> None:
    build_synth()
    build_cuda()
    build_cli()
