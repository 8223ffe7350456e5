"""Builds libcambgpu.so (CUDA for sm_103a + host C++) in-tree with nvcc.

The product library is `camb_gb300/_build/libcambgpu.so`; it is built from the
sources under `camb_gb300/csrc` with one `-gencode` for sm_103a.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcambgpu.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["ode_thread_a.cu", "ode_thread_b.cu", "ode_thread_c.cu", "ode_thread_d.cu", "ode_thread_e.cu",
              "ode_warp.cu",
              "ode_kernel.cu", "los_kernel.cu", "cl_lensing.cu", "capi.cu", "noalloc.cu", "tc_gemm.cu", "tc_proj.cu"]
TEMPLATE = os.path.join(HERE, "data", "highl_template.f64")
CXX_SOURCES = ["host/cosmo_host.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _template_source(path):
    """C++ source holding the high-L template table (data/highl_template.f64) as hex floats."""
    import struct
    raw = open(TEMPLATE, "rb").read()
    vals = struct.unpack("<%dd" % (len(raw) // 8), raw)
    assert len(vals) == 8001 * 4
    body = ",\n".join(", ".join(float(v).hex() for v in vals[i:i + 8]) for i in range(0, len(vals), 8))
    with open(path, "w") as f:
        f.write("namespace cgdev {\nextern const double kHighLTemplate[8001 * 4];\n"
                "const double kHighLTemplate[8001 * 4] = {\n" + body + "};\n}\n")


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CXX_SOURCES]
    hdrs = []
    for root, _, files in os.walk(CSRC):
        hdrs += [os.path.join(root, f) for f in files if f.endswith((".cuh", ".hpp", ".h"))]
    hdrs.append(os.path.join(HERE, "..", "include", "cambgpu.h"))
    hdrs.append(TEMPLATE)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) < t for f in srcs + hdrs):
            return LIB
    objs = []
    cmds = []
    for s in CU_SOURCES:
        o = os.path.join(BUILD, s.replace("/", "_") + ".o")
        objs.append(o)
        cmds.append([NVCC, *GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-v" if verbose else "-O3", "-c", os.path.join(CSRC, s), "-o", o])
    for s in CXX_SOURCES:
        o = os.path.join(BUILD, s.replace("/", "_") + ".o")
        objs.append(o)
        cmds.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c",
                     os.path.join(CSRC, s), "-o", o])
    tsrc = os.path.join(BUILD, "highl_template.cpp")
    _template_source(tsrc)
    objs.append(os.path.join(BUILD, "highl_template.o"))
    cmds.append(["g++", "-O1", "-std=c++17", "-fPIC", "-c", tsrc, "-o", objs[-1]])
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    _run([NVCC, *GENCODE, "-shared", "-o", LIB + ".tmp", *objs, "-lpthread"])
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
