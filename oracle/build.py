"""Builds the host oracle (test infrastructure) into oracle/lib/liboracle_mgpu.so.

Only tests, the smoke check and bench.py's CPU-baseline leg load this library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["oracle.cpp", "ref_emulation.cpp"]
LIB = os.path.join(HERE, "lib", "liboracle_mgpu.so")


def build(force=False):
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-o", LIB] + srcs
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
