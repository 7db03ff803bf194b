"""Builds the oracle's shared library (TEST INFRASTRUCTURE ONLY).

The oracle is the FP64 CPU restatement in isar_oracle.c.  It is compiled with
the host gcc on whatever machine runs the tests (x86_64 here, aarch64 on the
GPU host), into oracle/_build/liboracle.so.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRCS = [os.path.join(HERE, "isar_oracle.c")]


def build(force=False, quiet=True):
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SRCS + [os.path.join(HERE, "isar_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-o", tmp] + SRCS + ["-lm"]
    if not quiet:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, quiet=False))
