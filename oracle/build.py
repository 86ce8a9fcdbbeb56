"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/soda_oracle.c into oracle/_build/liboracle.so with gcc,
OpenMP and -ffp-contract=off (no fused multiply-add, so x86-64 and aarch64
hosts round the same way).
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = [os.path.join(HERE, "soda_oracle.c")]
DEPS = SRC + [os.path.join(HERE, "soda_oracle.h"), os.path.join(HERE, "..", "include", "sodagpu.h")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    cmd = [cc, "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wno-unused-function", "-o", LIB] + SRC + ["-lm"]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
