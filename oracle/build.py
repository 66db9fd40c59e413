"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/cunfft_oracle.c`` into ``oracle/liboracle.so`` with gcc and
OpenMP.  ``-ffp-contract=off`` keeps the floating-point results identical on
x86_64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cunfft_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")


def build_oracle(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11",
           "-shared", "-fPIC", "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
