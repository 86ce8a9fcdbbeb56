"""Build step for libsodagpu.so (the sm_103a C-ABI library) and the host CLI.

Every translation unit is compiled in parallel with nvcc for sm_103a only and
linked in-tree: sodabayes_gb300/libsodagpu.so, sodabayes_gb300/sodabayes.
Run as `python -m sodabayes_gb300.build` or through __graft_entry__.build().
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
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsodagpu.so")
CLI = os.path.join(PKG, "sodabayes")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["api.cu", "zbuild.cu", "sweep.cu", "noalloc.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libsodagpu.so")
    return cand


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build command failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    if proc.stdout.strip() and os.environ.get("SODAGPU_BUILD_VERBOSE"):
        sys.stderr.write(proc.stdout)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "sodagpu.h"))
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                    "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
    if verbose:
        flags += ["-Xptxas", "-v"]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nv] + flags + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    if force or _stale(LIB, objs):
        _run([nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    cli_src = os.path.join(CSRC, "host", "sodabayes_main.cpp")
    if os.path.exists(cli_src):
        host_srcs = [os.path.join(CSRC, "host", f) for f in sorted(os.listdir(os.path.join(CSRC, "host")))
                     if f.endswith(".cpp")]
        if force or _stale(CLI, host_srcs + [LIB] + headers):
            gxx = shutil.which("g++") or "g++"
            _run([gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-o", CLI] + host_srcs +
                 ["-L" + PKG, "-lsodagpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
