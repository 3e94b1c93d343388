"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/vfps_oracle.cpp into oracle/_build/libvfps_oracle.so with
-ffp-contract=off, so that the float restatement rounds like the reference
CPU build on both x86-64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "vfps_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvfps_oracle.so")


def build(force=False):
    """Compile the oracle shared library if it is missing or stale."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread",
           "-ffp-contract=off", "-fno-fast-math", SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
