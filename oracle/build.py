"""Build the CPU oracle (test infrastructure) into oracle/_build/.

g++ -O2, no -march tuning, -ffp-contract=off (the float pickers must round
like the reference). The reference itself is Rust and cannot be built here
(no Rust toolchain), so there is no oracle/_ref build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libzforacle.so")
SRC = [os.path.join(HERE, "zf_oracle.cpp")]
DEPS = SRC + [os.path.join(HERE, "zf_oracle.h"), os.path.join(HERE, "..", "include", "zf_filter.h"),
              os.path.join(HERE, "..", "include", "zf_av1_tables.h")]


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp] + SRC
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
