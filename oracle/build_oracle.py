"""Build recipe for the CPU oracle shared library (test infrastructure only).

Compiles ``oracle/effsc_oracle.c`` into ``oracle/_build/liboracle.so`` with
OpenMP.  Only the tests, the smoke check and the CPU-baseline leg of the
benchmark load the result.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "effsc_oracle.c")
    hdr = os.path.join(HERE, "effsc_oracle.h")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-Wall",
           "-Wno-unknown-pragmas", src, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
