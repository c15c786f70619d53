"""TEST INFRASTRUCTURE ONLY: ctypes view of liboracle.so (the CPU oracle).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module, as the checker or the timed CPU baseline; the product never does.
"""
import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DAG = os.path.join(HERE, "_ref", "ref_dag")


class CholArgs(ctypes.Structure):
    _fields_ = [("n_threads", ctypes.c_int), ("block_size", ctypes.c_int), ("num_blocks", ctypes.c_int),
                ("prio_kind", ctypes.c_int), ("accumulate", ctypes.c_int), ("upper_block_size", ctypes.c_int),
                ("matrix", ctypes.c_int), ("alpha", ctypes.c_double), ("seed", ctypes.c_uint32),
                ("record_dag", ctypes.c_int), ("dag_prefix", ctypes.c_char_p), ("panel_limit", ctypes.c_int),
                ("in_tiles", ctypes.c_void_p)]


class CholOut(ctypes.Structure):
    _fields_ = [("L", ctypes.c_void_p), ("A", ctypes.c_void_p), ("time_s", ctypes.c_double), ("potrf_s", ctypes.c_double),
                ("trsm_s", ctypes.c_double), ("gemm_s", ctypes.c_double), ("accu_s", ctypes.c_double),
                ("flops", ctypes.c_double), ("n_tasks_run", ctypes.c_long), ("n_edges", ctypes.c_long), ("errors", ctypes.c_long), ("info", ctypes.c_int),
                ("blas", ctypes.c_char * 256)]


class GemmArgs(ctypes.Structure):
    _fields_ = [("n_threads", ctypes.c_int), ("matrix_size", ctypes.c_int), ("block_size", ctypes.c_int),
                ("inputs", ctypes.c_int), ("seed", ctypes.c_uint32), ("record_dag", ctypes.c_int),
                ("dag_prefix", ctypes.c_char_p)]


class GemmOut(ctypes.Structure):
    _fields_ = [("C", ctypes.c_void_p), ("time_s", ctypes.c_double), ("n_tasks_run", ctypes.c_long),
                ("n_edges", ctypes.c_long), ("errors", ctypes.c_long), ("blas", ctypes.c_char * 256)]


def build():
    """Build liboracle.so, and oracle/_ref when the reference tree is present
    (the Makefile's REF, or TTG_REFERENCE_DIR when set)."""
    subprocess.run(["make", "-s", "liboracle.so"], cwd=HERE, check=True)
    ref = os.environ.get("TTG_REFERENCE_DIR")
    cmd = ["make", "-s", "ref-if-present"] + (["REF=" + ref] if ref else [])
    subprocess.run(cmd, cwd=HERE, check=True)


def find_openblas():
    """Path of the OpenBLAS shipped in the scipy wheel (32-bit integers), or None."""
    try:
        import scipy
    except ImportError:
        return None
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    for pat in ("scipy.libs/libscipy_openblas-*.so", "scipy.libs/libopenblas*.so"):
        hits = sorted(glob.glob(os.path.join(base, pat)))
        if hits:
            return hits[0]
    return None


_lib = None


def lib(use_blas=False):
    """Load liboracle.so.  use_blas=True points the oracle's tile math at the
    host OpenBLAS (must be decided before the first load)."""
    global _lib
    if _lib is None:
        if use_blas:
            p = find_openblas()
            if p:
                os.environ["TTG_ORACLE_BLAS"] = p
        else:
            os.environ.pop("TTG_ORACLE_BLAS", None)
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_cholesky.argtypes = [ctypes.POINTER(CholArgs), ctypes.POINTER(CholOut)]
        L.orc_gemm.argtypes = [ctypes.POINTER(GemmArgs), ctypes.POINTER(GemmOut)]
        L.orc_blas_name.restype = ctypes.c_char_p
        L.orc_gen_gram.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_uint32, ctypes.c_void_p]
        L.orc_block_sizes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.orc_gemm_inputs.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
        for f in ("orc_normals", "orc_uniforms", "orc_qnormals"):
            getattr(L, f).argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
        L.orc_philox.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_gram_entry.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_uint32]
        L.orc_gram_entry.restype = ctypes.c_double
        _lib = L
    return _lib


def blas_name():
    return lib().orc_blas_name().decode()


def cholesky(N=None, block_size=32, num_blocks=8, n_threads=4, kind=0, accumulate=False, upper_block_size=-1, matrix=1,
             alpha=1.0, seed=0, want_L=True, want_A=False, dag_prefix=None, panel_limit=0, tiles=None):
    """One run of the oracle's Cholesky task graph.  Returns a dict.

    tiles: the input as packed lower tiles (float64, the device layout of
    ttg_tile_layout); sets matrix = 2.  panel_limit > 0 runs only the tasks
    of the first panel_limit panel steps (a bounded sample; `flops` counts
    the tasks that ran)."""
    sizes = block_sizes(block_size, num_blocks, upper_block_size)
    n = int(sizes.sum())
    L = np.zeros((n, n), order="F") if want_L else None
    A = np.zeros((n, n), order="F") if want_A else None
    tp = None
    if tiles is not None:
        matrix = 2
        tiles = np.ascontiguousarray(tiles, dtype=np.float64)
        need = sum(int(sizes[i]) * int(sizes[j]) for j in range(num_blocks) for i in range(j, num_blocks))
        if tiles.size < need:
            raise ValueError("tiles: %d elements, the layout needs %d" % (tiles.size, need))
        tp = tiles.ctypes.data
    a = CholArgs(n_threads, block_size, num_blocks, kind, 1 if accumulate else 0, upper_block_size, matrix, alpha, seed,
                 1 if dag_prefix else 0, dag_prefix.encode() if dag_prefix else None, panel_limit, tp)
    o = CholOut(L.ctypes.data if L is not None else None, A.ctypes.data if A is not None else None)
    r = lib().orc_cholesky(ctypes.byref(a), ctypes.byref(o))
    if r != 0:
        raise RuntimeError("orc_cholesky failed")
    return {"L": L, "A": A, "time_s": o.time_s, "flops": o.flops, "tasks": o.n_tasks_run, "edges": o.n_edges, "errors": o.errors,
            "info": o.info, "blas": o.blas.decode(), "N": n,
            "kind_s": {"potrf": o.potrf_s, "trsm": o.trsm_s, "gemm": o.gemm_s, "accu": o.accu_s}}


def gemm(N, block_size, n_threads=4, inputs=1, seed=1, want_C=True, dag_prefix=None):
    C = np.zeros((N, N), order="F") if want_C else None
    a = GemmArgs(n_threads, N, block_size, inputs, seed, 1 if dag_prefix else 0, dag_prefix.encode() if dag_prefix else None)
    o = GemmOut(C.ctypes.data if C is not None else None)
    r = lib().orc_gemm(ctypes.byref(a), ctypes.byref(o))
    if r != 0:
        raise RuntimeError("orc_gemm failed")
    return {"C": C, "time_s": o.time_s, "tasks": o.n_tasks_run, "edges": o.n_edges, "errors": o.errors,
            "blas": o.blas.decode()}


def gram(N, alpha, seed):
    A = np.zeros((N, N), order="F")
    lib().orc_gen_gram(N, alpha, seed, A.ctypes.data)
    return A


def gram_entry(N, i, j, alpha, seed):
    """Entry (i, j) of A = G·Gᵀ/N + αI, computed on its own."""
    return lib().orc_gram_entry(N, i, j, alpha, seed)


def gemm_inputs(N, inputs, seed):
    A = np.zeros((N, N), order="F")
    B = np.zeros((N, N), order="F")
    lib().orc_gemm_inputs(N, inputs, seed, A.ctypes.data, B.ctypes.data)
    return A, B


def block_sizes(block_size, num_blocks, upper_block_size=-1):
    out = np.zeros(num_blocks, dtype=np.int32)
    if lib().orc_block_sizes(block_size, num_blocks, upper_block_size, out.ctypes.data) != 0:
        raise ValueError("bad block sizes")
    return out


def normals(first, count, seed, stream):
    out = np.zeros(count)
    lib().orc_normals(first, count, seed, stream, out.ctypes.data)
    return out


def uniforms(first, count, seed, stream):
    out = np.zeros(count)
    lib().orc_uniforms(first, count, seed, stream, out.ctypes.data)
    return out


def qnormals(first, count, seed, stream):
    out = np.zeros(count, dtype=np.int32)
    lib().orc_qnormals(first, count, seed, stream, out.ctypes.data)
    return out


def philox(ctr, key):
    c = np.array(ctr, dtype=np.uint32)
    k = np.array(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox(c.ctypes.data, k.ctypes.data, o.ctypes.data)
    return [int(x) for x in o]


def read_dag(prefix):
    """(tasks: {name: (indegree, promises, runs)}, sorted edge list) of a DAG record."""
    import gzip
    def _open(p):
        return gzip.open(p, "rt") if p.endswith(".gz") else open(p)
    sfx = ".gz" if os.path.exists(prefix + ".tasks.csv.gz") else ""
    tasks = {}
    with _open(prefix + ".tasks.csv" + sfx) as f:
        next(f)
        for line in f:
            n, i, p, r = line.strip().split(",")
            tasks[n] = (int(i), int(p), int(r))
    with _open(prefix + ".edges.csv" + sfx) as f:
        edges = sorted(tuple(l.strip().split(",")) for l in f if l.strip())
    return tasks, edges
