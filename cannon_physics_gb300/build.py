"""Builds libcannon_gpu.so in-tree for sm_103a (GB300).

nvcc compiles the step kernels and the host runtime in parallel, with
-fmad=false (no fused multiply-add on the device) and -ffp-contract=off on
the host: the reference never fuses a multiply and an add, and parity is
bit-exact.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcannon_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

DEVICE_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-ftz=false", "-prec-div=true", "-prec-sqrt=true",
                "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I" + os.path.join(ROOT, "include")]

UNITS = ["cp_step.cu", "cp_wide.cu", "cp_ray.cu", "cp_host.cpp", "cp_serve.cpp"]


def _sources():
    return [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(ROOT, "include", "cannon_gpu.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _sources())


def _compile(unit, verbose):
    src = os.path.join(SRC, unit)
    obj = os.path.join(OUT_DIR, unit + ".o")
    cmd = [NVCC] + ARCH + DEVICE_FLAGS + ["-c", src, "-o", obj]
    if verbose and unit.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with ThreadPoolExecutor(len(UNITS)) as ex:
        results = list(ex.map(lambda u: _compile(u, verbose), UNITS))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                print(err)
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
