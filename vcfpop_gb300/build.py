"""Build the in-tree CUDA library (and the command-line driver) for sm_103a.

nvcc compiles every translation unit in parallel; outputs stay next to the
sources' package (vcfpop_gb300/libvcfpop_structure.so, vcfpop_gb300/vcfpop-gb300)
and are git-ignored.
"""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libvcfpop_structure.so")
CLI = os.path.join(PKG, "vcfpop-gb300")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: the reference-stream kernels must round like the reference's
# -ffp-contract=off build; hot loops that want FMA use explicit intrinsics.
FLAGS = ["-O3", "--fmad=false", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"] + ARCH

CU = ["vp_structure.cu", "vp_ingest.cu"]
CPP = ["vp_data.cpp", "vp_server.cpp", "vp_write.cpp"]  # vp_cli.cpp is the driver binary, built with g++ below


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False):
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    if not os.path.exists(CLI):
        deps.append(CLI)
    deps.append(os.path.join(os.path.dirname(PKG), "include", "vcfpop_structure.h"))
    if os.path.exists(CLI) and not _newer(LIB, deps) and not _newer(CLI, deps):
        return LIB
    objdir = os.path.join(PKG, "_build")
    os.makedirs(objdir, exist_ok=True)
    procs, objs = [], []
    for f in CU + CPP:
        o = os.path.join(objdir, f + ".o")
        objs.append(o)
        cmd = [NVCC] + FLAGS + ["-c", os.path.join(CSRC, f), "-o", o]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode())
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
        if verbose:
            sys.stderr.write(out.decode())
    tmp = LIB + ".tmp"
    subprocess.check_call([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    # the command-line driver links the library by its in-tree path
    cli_obj = os.path.join(objdir, "vp_cli.o")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-c", os.path.join(CSRC, "vp_cli.cpp"), "-o", cli_obj])
    subprocess.check_call(["g++", "-o", CLI, cli_obj, LIB, "-Wl,-rpath," + PKG, "-lz"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
