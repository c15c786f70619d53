"""Build the native parts in-tree: libttg.so (CUDA executor, tile kernels,
C ABI, miniapp plans) and the 2d_cholesky / 2d_gemm command-line programs.

All device code is compiled for sm_103a only.  Host code is compiled with
-ffp-contract=off so that the seeded input generator gives the same bits on
the host and the device.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(HERE, "libttg.so")
BIN = os.path.join(HERE, "bin")

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
CUDA_HOME = os.path.dirname(os.path.dirname(os.path.realpath(NVCC)))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]

CU_SOURCES = ["ttg_exec.cu", "ttg_gen.cu", "ttg_mixed.cu", "ttg_solve.cu", "ttg_sliced.cu", "ttg_noalloc.cu", "ttg_batch.cu",
              "ttg_serve.cu"]
CPP_SOURCES = ["apps.cpp"]
MINIAPPS = ["2d_cholesky.cpp", "2d_gemm.cpp", "ttor_wait.cpp", "ttor_deps.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = []
    for d in (CSRC, os.path.join(ROOT, "include"), os.path.join(HERE, "tasktorrent"), os.path.join(HERE, "tasktorrent", "src")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                hs.append(os.path.join(d, f))
    return hs


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    headers = _headers()
    cmds = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            cmds.append([NVCC] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            cmds.append(["g++"] + HOST_FLAGS + ["-I", os.path.join(CUDA_HOME, "include"), "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or max(2, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if _newer(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    # Command-line programs with the reference's flags.
    progs = []
    for src in MINIAPPS:
        s = os.path.join(HERE, "miniapp", src)
        exe = os.path.join(BIN, src[:-4])
        if _newer(exe, [s, LIB] + headers):
            progs.append(["g++"] + HOST_FLAGS + ["-I", os.path.join(CUDA_HOME, "include"), s, "-o", exe,
                          "-L", HERE, "-lttg", "-Wl,-rpath,$ORIGIN/..", "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart"])
    with cf.ThreadPoolExecutor(max_workers=len(progs) or 1) as ex:
        list(ex.map(_run, progs))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
