"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/cannon_oracle.cpp into oracle/_build/liboracle.so with
-ffp-contract=off so that no multiply-add is fused (the reference, Dart,
never fuses).  The reference itself is Dart + Flutter and has no C sources to
compile, so there is no oracle/_ref build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "cannon_oracle.cpp")
    hdrs = [os.path.join(HERE, "cannon_oracle.h"), os.path.join(ROOT, "include", "cannon_gpu.h")]
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(p) for p in [src] + hdrs)
        if os.path.getmtime(OUT) >= newest:
            return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-I" + os.path.join(ROOT, "include"), "-o", OUT + ".tmp", src, "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
