"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/mlegs_oracle.cpp into oracle/liboracle.so with the host's g++.  The oracle is the
parity checker and the CPU baseline; the product never links it.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mlegs_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")


def build(force=False, verbose=False):
    hdr = os.path.join(HERE, "..", "include", "mlegs_gb300.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB + ".tmp", SRC]
    if platform.machine() in ("x86_64", "AMD64"):
        cmd.append("-lquadmath")
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
