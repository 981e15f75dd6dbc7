"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/cans_oracle.c into oracle/_build/libcans_oracle.so with gcc.
`-ffp-contract=off` keeps gcc from fusing a*b+c into FMAs (gcc's default on
aarch64), so the oracle gives the same bits on x86_64 and on Arm hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcans_oracle.so")
SRC = os.path.join(HERE, "cans_oracle.c")
HDR = os.path.join(HERE, "cans_oracle.h")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-variable", "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
