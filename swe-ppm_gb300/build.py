"""Builds the library in-tree: swe-ppm_gb300/_build/libswe_gb300.so.

CUDA sources are compiled for sm_103a only (one -gencode), in parallel, with
-fmad=false (every fused multiply-add in the kernels is an explicit fmaf) and
IEEE division / square root, so the kernels reproduce the CPU restatement bit
for bit.  The fast-arithmetic step (csrc/swe_fast.cu) is the exception: it is
compiled with contraction and approximate division / square root.  Host C++ (scenarios, initialisation, writer) is compiled with g++
-ffp-contract=off and linked into the same shared library.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libswe_gb300.so")
DRIVER = os.path.join(OUT, "swe_gb300")

CUDA_SOURCES = ["csrc/swe_capi.cu", "csrc/swe_kernels_fh.cu", "csrc/swe_kernels_aug.cu", "csrc/swe_lts.cu", "csrc/swe_mlp.cu",
                "csrc/swe_fast.cu"]
# the fast-arithmetic step (SWE_ARITH_FAST) is its own translation unit with
# contraction and approximate division and square root
FAST_SOURCES = {"csrc/swe_fast.cu"}
FAST_FLAGS = ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
HOST_SOURCES = ["host/swe_host.cpp", "host/netcdf_writer.cpp"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + os.path.join(ROOT, "include"),
             "-I" + os.path.join(HERE, "host")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps():
    out = []
    for sub in ("csrc", "host"):
        d = os.path.join(HERE, sub)
        out += [os.path.join(d, f) for f in os.listdir(d)]
    out += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return out


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB, deps) and not _stale(DRIVER, deps):
        return LIB
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        flags = NVCC_FLAGS
        if src in FAST_SOURCES:
            flags = [f for f in NVCC_FLAGS if f != "-fmad=false"] + FAST_FLAGS
        jobs.append([nvcc] + flags + ["-c", os.path.join(HERE, src), "-o", obj])
    for src in HOST_SOURCES:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        jobs.append(["g++"] + CXX_FLAGS + ["-c", os.path.join(HERE, src), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("compilation failed: " + " ".join(cmd))

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    run([nvcc, "-shared", "-o", LIB] + objs + ["-lcudart"])
    # the driver executable (reference drivers' flags), linked against the library
    run(["g++"] + CXX_FLAGS + ["-o", DRIVER, os.path.join(HERE, "host", "swe_gb300_main.cpp"), "-L" + OUT,
                               "-lswe_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
