"""Build recipe for the CPU oracle (test infrastructure, not the product).

Compiles oracle/oracle.c into oracle/_build/liboracle.so with gcc + OpenMP.
-ffp-contract=off keeps the results bit-identical between x86_64 and aarch64
hosts, so the committed golden fixtures compare exactly on both.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= os.path.getmtime(src):
        return SO
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O3", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", SO + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(SO + ".tmp", SO)
    return SO


if __name__ == "__main__":
    print(build(force=True))
