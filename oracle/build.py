"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle.c into oracle/_build/liboracle.so with gcc.  The flags keep
floating-point evaluation in source order (-ffp-contract=off, no fast-math),
so x86_64 and aarch64 hosts produce identical results.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-pthread", "-Wall", "-Wno-unused-function",
           src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
