"""Build recipe for the CPU oracle (test infrastructure, not the product).

Compiles oracle/craystal_oracle.cpp into oracle/_build/liboracle.so with
``-O2 -ffp-contract=off -fno-fast-math`` so that no multiply-add is fused and
the float arithmetic is the reference source's, on x86-64 and aarch64 alike.

The reference itself (Hyiker/CRaystal) is not compiled: every source file of
its hot path includes glm, which its CMake fetches from the network, so there
is no ``oracle/_ref`` build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "craystal_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")

FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-fPIC",
         "-shared", "-pthread", "-Wall", "-Wno-unused-function"]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = [SRC, os.path.join(HERE, "craystal_oracle.h"), os.path.abspath(__file__)]
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", *FLAGS, SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
