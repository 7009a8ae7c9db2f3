"""Build libsister_gb300.so in-tree for sm_103a with nvcc (translation units compiled in parallel), and the
headless CLI sister_compute_disp (host C++ over the library's C ABI).

    python -m sister_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsister_gb300.so")
CLI_SRC = os.path.join(CSRC, "cli")
CLI = os.path.join(HERE, "sister_compute_disp")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _flags(extra: list[str] | None = None) -> list[str]:
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                   "-I", CSRC, "-I", os.path.join(ROOT, "include")] + (extra or [])


def _cli_sources() -> list[str]:
    return sorted(os.path.join(CLI_SRC, f) for f in os.listdir(CLI_SRC) if f.endswith((".cpp", ".h")))


def build_cli(force: bool = False) -> str:
    """sister_compute_disp, linked against the in-tree library (rpath $ORIGIN)."""
    srcs = _cli_sources()
    newest = max(os.path.getmtime(p) for p in srcs + [LIB, __file__, os.path.join(ROOT, "include", "sister_gb300.h")])
    if not force and os.path.exists(CLI) and os.path.getmtime(CLI) >= newest:
        return CLI
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = CLI + ".tmp.%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", CLI_SRC] + \
          [p for p in srcs if p.endswith(".cpp")] + ["-L", HERE, "-lsister_gb300", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s%s" % (p.stdout, p.stderr))
    os.replace(tmp, CLI)
    return CLI


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    lib = build_lib(force, verbose, ptxas_info)
    build_cli(force)
    return lib


def build_lib(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    srcs = sources()
    newest_dep = max(os.path.getmtime(p) for p in srcs + _headers() + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest_dep:
        return LIB
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src: str) -> tuple[str, str]:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc] + _flags(extra) + ["-c", src, "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, p.stdout, p.stderr))
        return obj, p.stdout + p.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose or ptxas_info:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (p.stdout, p.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
