"""Build the CPU oracle (test infrastructure only).

Compiles ``oracle/e2d_oracle.c`` into ``oracle/liboracle.so`` with gcc and
OpenMP.  ``-ffp-contract=off`` keeps every multiply and add a separate IEEE
operation on both x86-64 and aarch64 (gcc fuses them by default on aarch64),
which the bit-exact FP64 parity checks rely on.

Usage: ``python oracle/build.py``.  The library is loaded only by ``tests/``,
``__graft_entry__.smoke()`` and the cpu_baseline leg of ``bench.py``.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "e2d_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

CFLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas"]


def build(force: bool = False) -> str:
    hdr = os.path.join(HERE, "e2d_oracle.h")
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(SRC), os.path.getmtime(hdr))
        if os.path.getmtime(LIB) >= newest:
            return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", *CFLAGS, SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
