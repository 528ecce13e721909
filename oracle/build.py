"""Build recipe for the oracle library (test infrastructure only).

Compiles oracle/geon_oracle.cpp with g++ into oracle/_build/libgeon_oracle.so.
-ffp-contract=off keeps a*b+c unfused, as Rust evaluates it; no fast-math.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgeon_oracle.so")
SRC = os.path.join(HERE, "geon_oracle.cpp")
HDR = os.path.join(HERE, "geon_oracle.h")

CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            "-pthread"]


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR), os.path.getmtime(__file__))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", *CXXFLAGS, SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
