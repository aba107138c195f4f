"""Build recipe for the CPU oracle (test infrastructure).

Compiles ``fem_oracle.cpp`` with the system C++ compiler into
``oracle/_build/libfem_oracle.so``.  Portable flags only (the same source
builds on x86_64 and aarch64 hosts); FP64 without fast-math so that the
oracle keeps IEEE semantics.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfem_oracle.so")


def build(force=False):
    src = os.path.join(HERE, "fem_oracle.cpp")
    hdr = os.path.join(HERE, "fem_oracle.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(src), os.path.getmtime(hdr))
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["g++", "-O3", "-std=c++20", "-fPIC", "-shared", "-pthread", "-fno-fast-math",
           "-ffp-contract=off", src, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
