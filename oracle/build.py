"""Build recipe for the oracle library (test infrastructure only).

Compiles oracle/icsref.cpp into oracle/libicsref.so with -ffp-contract=off so
that x86 and Arm hosts produce identical floating-point results.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libicsref.so")
SRC = os.path.join(HERE, "icsref.cpp")


def build(force: bool = False) -> str:
    hdr = os.path.join(HERE, "..", "include", "icsfoam_gb300.h")
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(SRC), os.path.getmtime(hdr))
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-o", LIB + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def popen_build():
    """Start the compile asynchronously; returns the Popen (or None if up to date)."""
    hdr = os.path.join(HERE, "..", "include", "icsfoam_gb300.h")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr)):
        return None
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-o", LIB, SRC]
    return subprocess.Popen(cmd)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
