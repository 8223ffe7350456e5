"""ORACLE -- test infrastructure only.  Builds oracle/_build/liboracle.so from
camb_oracle.cpp and lensing_oracle.cpp with g++ and OpenMP (the reference's own
parallelism)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRCS = [os.path.join(HERE, "camb_oracle.cpp"), os.path.join(HERE, "lensing_oracle.cpp")]
HDR = os.path.join(HERE, "..", "include", "cambgpu.h")


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > max(os.path.getmtime(f) for f in SRCS + [HDR]):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", *SRCS, "-o", LIB + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
