"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/sv_oracle.c`` into ``oracle/liboracle.so`` with gcc and OpenMP.
``-ffp-contract=off -fcx-limited-range`` keep the arithmetic identical to the
reference's plain-Python complex products (no fused multiply-add, no C99 Annex G
special-casing).  Portable flags only: the same recipe runs on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sv_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = [
        "gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fcx-limited-range", "-fno-fast-math",
        SRC, "-o", LIB + ".tmp", "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
