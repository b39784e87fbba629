"""Build the native library libshl_gb300.so in-tree (shell_gb300/_build/).

CUDA sources are compiled for sm_103a only; host sources with g++.  Every host
translation unit is compiled with -ffp-contract=off: the contact geometry
shared with the device (csrc/shl_geom.h) must round each multiply and add on
its own, as the device code does with __dmul_rn/__dadd_rn.

Usage:  python -m shell_gb300.build [--force]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libshl_gb300.so")
RUN = os.path.join(OUT, "shl_run")  # the command-line driver (csrc/shl_run.cpp)

CU_SOURCES = ["shl_kernels.cu", "shl_contact.cu", "shl_api.cu", "shl_mlp.cu"]
CPP_SOURCES = ["shl_setup.cpp", "shl_host.cpp", "shl_io.cpp"]
HEADERS = ["shl_geom.h", "shl_distance.h", "shl_limit.h", "shl_setup.h", "shl_internal.cuh", "shl_expr.h", "shl_smooth.h", "shl_subdiv.h",
           os.path.join("..", "..", "include", "shl.h")]

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                     "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-g", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall",
             "-Wno-unused-function"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile and link; returns the path of the shared library."""
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([CXX] + CXX_FLAGS + ["-I", os.path.join(CUDA_HOME(), "include"), "-c", s, "-o", o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append((j, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + out for j, out in failed)
        raise RuntimeError("libshl_gb300 build failed:\n" + msg)
    if force or jobs or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout.decode(errors="replace"))
    run_src = os.path.join(CSRC, "shl_run.cpp")
    if force or _stale(RUN, [run_src, LIB] + headers):
        cmd = [CXX] + [f for f in CXX_FLAGS if f != "-fPIC"] + ["-o", RUN, run_src, "-L", OUT, "-lshl_gb300",
                                                                "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("driver build failed:\n" + " ".join(cmd) + "\n" + r.stdout.decode(errors="replace"))
    return LIB


def CUDA_HOME():
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
