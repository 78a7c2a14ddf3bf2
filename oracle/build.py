"""Builds the CPU restatement (oracle/nl_oracle.cpp) into oracle/liborc.so.

Test infrastructure only.  Portable flags (no ISA-specific options) so the same
recipe works on x86-64 and aarch64 hosts; -ffp-contract=off keeps the
arithmetic order of the reference (no fused multiply-add contraction).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nl_oracle.cpp")
LIB = os.path.join(HERE, "liborc.so")


def build(force: bool = False) -> str:
    deps = [SRC, os.path.join(HERE, "eigen_shim", "Eigen", "src", "shim.hpp")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-std=c++20", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I", HERE, SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
