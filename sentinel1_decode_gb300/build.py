"""Build the in-tree CUDA library libs1g.so for sm_103a with nvcc.

Every translation unit is compiled in parallel into _build/, then linked into
one shared library exposing the C ABI of include/s1g.h.  No CMake, no torch
extension machinery: plain nvcc, so the same recipe runs on x86 (cross
compile, no GPU needed) and on the Arm GPU host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libs1g.so")
CLI = os.path.join(OUT, "s1g_write")
CLI_SRC = os.path.join(HERE, "cli", "s1g_write.cpp")
PRINT_CLI = os.path.join(OUT, "s1g_print")
PRINT_CLI_SRC = os.path.join(HERE, "cli", "s1g_print.cpp")
INCLUDE = os.path.join(HERE, "..", "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["s1g_fft_engine.cu", "s1g_tune.cu", "s1g_decode.cu", "s1g_sar.cu", "s1g_fast.cu", "s1g_dcest.cu", "s1g_image.cu", "s1g_adjoint.cu", "s1g_api.cu", "s1g_noalloc.cu", "s1g_sinc.cu", "s1g_tma.cu", "s1g_eccm.cu", "s1g_model.cpp", "s1g_aux.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(SRC, src)
    deps = [path] + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "s1g.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    # host code without floating-point contraction: the host arithmetic that
    # restates the reference's (state vectors, attitudes, geometry) rounds
    # the same way on x86-64 and aarch64
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off", "-c", path, "-o", obj,
           "-I", SRC, *extra]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off", "-c", path, "-o", obj, "-I", SRC,
               "-x", "cu", *ARCH]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    return obj


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(SRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
    build_cli()
    if verbose:
        print("built", LIB, CLI, PRINT_CLI)
    return LIB


def _build_tool(out: str, src: str, deps) -> str:
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in [src, LIB, *deps]):
        return out
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, src, "-o", out, "-L", OUT, "-ls1g", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s build failed:\n%s\n%s" % (os.path.basename(out), " ".join(cmd), r.stderr[-4000:]))
    return out


def build_cli() -> str:
    """The command-line tools, host C++ linked against libs1g.so: s1g_write
    (the reference's s1_write commands, over the facade header
    include/s1_decoder_gb300.hpp) and s1g_print (its s1_print commands, over
    the C ABI)."""
    _build_tool(PRINT_CLI, PRINT_CLI_SRC, [os.path.join(INCLUDE, "s1g.h")])
    return _build_tool(CLI, CLI_SRC, [os.path.join(INCLUDE, "s1g.h"), os.path.join(INCLUDE, "s1_decoder_gb300.hpp")])


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
