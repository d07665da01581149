"""Builds the oracle (test infrastructure): oracle/_build/libt3d_oracle.so.

The restatement is compiled with -ffp-contract=off and without fast-math so it
evaluates the reference's arithmetic as unfused IEEE binary32 on both x86_64 and
aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libt3d_oracle.so")
SRCS = [os.path.join(HERE, "t3d_oracle.cpp"), os.path.join(HERE, "t3d_oracle_raster.cpp")]
DEPS = SRCS + [os.path.join(HERE, "t3d_oracle.h"), os.path.join(HERE, "..", "include", "t3d.h")]


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
           "-o", LIB, *SRCS]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
