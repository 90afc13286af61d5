"""In-tree build of the CUDA library (libocrt_gb300.so) for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked into a
shared library next to this file.  No cmake, no torch extension machinery:
the product is a plain C-ABI shared object.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libocrt_gb300.so")
SOURCES = ["setup.cu", "sos.cu", "post.cu", "api.cu", "noalloc.cu", "tc_gemm.cu", "adjoint.cu", "lut.cu",
           "coxmunk_tc.cu", "gas.cu", "ocean.cu", "scan_tma.cu", "mie.cu", "value.cu", "tables_tc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(HERE, "..", "include", "ocrt_gb300.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if _stale(o, s):
            jobs.append([nvcc, *ARCH, *FLAGS, *extra, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if jobs or not os.path.exists(LIB):
        run([nvcc, *ARCH, "-shared", *objs, "-o", LIB, "-lcudart"])
    build_cli(run)
    return LIB


CLI_SRC = os.path.join(HERE, "cli", "ocrt_cli.c")
CLI_BIN = os.path.join(HERE, "bin", "ocrt")


def build_cli(run):
    """The `ocrt` command-line front end: plain C over the C ABI."""
    if os.path.exists(CLI_BIN) and os.path.getmtime(CLI_BIN) >= max(os.path.getmtime(CLI_SRC), os.path.getmtime(LIB)):
        return CLI_BIN
    os.makedirs(os.path.dirname(CLI_BIN), exist_ok=True)
    run([os.environ.get("CC", "gcc"), "-std=c11", "-O2", "-Wall", "-Werror=implicit-function-declaration", CLI_SRC, "-I", os.path.join(HERE, "..", "include"),
         "-L", HERE, "-locrt_gb300", "-Wl,-rpath,$ORIGIN/..", "-lm", "-o", CLI_BIN])
    return CLI_BIN


if __name__ == "__main__":
    print(build(verbose=True, extra=tuple(sys.argv[1:])))
