"""Build libomni3d_gb300.so (and the omni3d command-line program) in-tree with nvcc.

Every CUDA translation unit is compiled for sm_103a only.  Objects are compiled in
parallel; the result goes to <package>/_build/.  Host code is compiled with
-ffp-contract=off so that the direction table and the icosphere are bit-identical on
x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libomni3d_gb300.so")
CLI = os.path.join(BUILD, "omni3d")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["kernels_trace.cu", "kernels_sweep.cu", "kernels_anchor.cu", "kernels_adjoint.cu", "kernels_brick.cu",
               "kernels_fixed.cu", "api.cu", "host_io.cpp", "noalloc.cu"]
CLI_SOURCES = ["cli.cpp"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libomni3d_gb300")


def _flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]


def _compile(src: str, obj: str) -> None:
    cmd = [_nvcc()] + ARCH + _flags() + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [_nvcc()] + _flags() + ["-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, cli: bool = True, jobs: int | None = None) -> str:
    """Compile the library (and the CLI); returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "omni3d.h"))
    todo = []
    objs = []
    for s in LIB_SOURCES + (CLI_SOURCES if cli else []):
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        if s in LIB_SOURCES:
            objs.append(obj)
        if force or _stale(obj, [src] + headers):
            todo.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_compile, s, o) for s, o in todo]:
            f.result()
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if cli:
        cobj = os.path.join(BUILD, "cli.cpp.o")
        if force or _stale(CLI, objs + [cobj]):
            tmp = CLI + ".tmp%d" % os.getpid()
            cmd = [_nvcc()] + ARCH + ["-o", tmp, cobj] + objs
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
            os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv))
