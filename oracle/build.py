"""Build recipe for the oracle (test infrastructure only).

Compiles ``oracle/nmmc_oracle.cpp`` into ``oracle/_build/libnmmc_oracle.so`` with g++.
``-ffp-contract=off`` keeps FP64 results independent of the host ISA (x86_64 here,
aarch64 on the GPU host). No ``-march=native``: the same flags must work on both.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nmmc_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnmmc_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
