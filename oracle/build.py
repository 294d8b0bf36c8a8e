"""Build recipe for the oracle's C restatement (test infrastructure only).

Compiles oracle/ed_oracle.c into oracle/_build/libedoracle.so with gcc.  OpenMP is
used when the compiler supports it (the CPU baseline then uses every host thread);
otherwise the library is built single-threaded.  The reference itself is Julia and
cannot be compiled here, so there is no oracle/_ref build.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ed_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libedoracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    base = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", SRC, "-o", LIB, "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True, capture_output=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
