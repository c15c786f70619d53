"""Python view of the GB300 task-graph executor (libttg.so).

The product is the C ABI (include/ttg.h, include/ttg_apps.h) and the C++
Taskflow<K> drop-in (tasktorrent_gb300/tasktorrent/).  This module binds the C
ABI with ctypes for the test suite, the smoke check and bench.py.  It loads the
in-tree libttg.so and raises if it is missing: there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libttg.so")
BIN_DIR = os.path.join(HERE, "bin")

# Status codes (include/ttg.h)
TTG_OK, TTG_EINVAL, TTG_ECUDA, TTG_ETIMEOUT, TTG_EOVERCOUNT, TTG_ENOTPD, TTG_ENOMEM, TTG_ESTATE, TTG_EUNDERRUN, TTG_ENOCONV = range(10)
# Tile operations
OP_NOP, OP_POTRF_L, OP_TRSM_RLTN, OP_SYRK_LN, OP_GEMM_NT, OP_GEMM_NN, OP_GEADD, OP_TRSM_RLNN, OP_CONVERT = range(9)
PREC_F64, PREC_MIXED = 0, 1


class TTGError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s: %s (status %d)" % (what, strerror(status), status))


class Op(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("prec", ctypes.c_int32), ("m", ctypes.c_int32), ("n", ctypes.c_int32),
                ("k", ctypes.c_int32), ("lda", ctypes.c_int32), ("ldb", ctypes.c_int32), ("ldc", ctypes.c_int32),
                ("parts", ctypes.c_int32), ("flags", ctypes.c_int32), ("alpha", ctypes.c_double), ("beta", ctypes.c_double), ("a", ctypes.c_void_p), ("b", ctypes.c_void_p),
                ("c", ctypes.c_void_p), ("aux", ctypes.c_void_p)]


class GraphDesc(ctypes.Structure):
    _fields_ = [("n_tasks", ctypes.c_int32), ("ops", ctypes.POINTER(Op)), ("init_count", ctypes.POINTER(ctypes.c_int32)),
                ("priority", ctypes.POINTER(ctypes.c_double)), ("bind", ctypes.POINTER(ctypes.c_int32)),
                ("succ_ptr", ctypes.POINTER(ctypes.c_int64)), ("succ_idx", ctypes.POINTER(ctypes.c_int32))]


class Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("workers", ctypes.c_int), ("timeout_s", ctypes.c_double), ("trace", ctypes.c_int)]


class Report(ctypes.Structure):
    _fields_ = [("tasks_total", ctypes.c_int64), ("tasks_run", ctypes.c_int64), ("tasks_pending", ctypes.c_int64),
                ("bad_runs", ctypes.c_int64), ("status", ctypes.c_int32), ("error_task", ctypes.c_int32),
                ("info", ctypes.c_int32), ("workers", ctypes.c_int32), ("elapsed_ms", ctypes.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class CholArgs(ctypes.Structure):
    _fields_ = [("n_threads", ctypes.c_int32), ("verb", ctypes.c_int32), ("block_size", ctypes.c_int32),
                ("num_blocks", ctypes.c_int32), ("kind", ctypes.c_int32), ("accumulate", ctypes.c_int32),
                ("upper_block_size", ctypes.c_int32), ("matrix", ctypes.c_int32), ("alpha", ctypes.c_double),
                ("seed", ctypes.c_uint32), ("precision", ctypes.c_int32), ("mixed_kind", ctypes.c_int32)]


class GemmArgs(ctypes.Structure):
    _fields_ = [("n_threads", ctypes.c_int32), ("verb", ctypes.c_int32), ("block_size", ctypes.c_int32),
                ("matrix_size", ctypes.c_int32), ("inputs", ctypes.c_int32), ("seed", ctypes.c_uint32)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("nrhs", ctypes.c_int32), ("tol", ctypes.c_double), ("max_outer", ctypes.c_int32),
                ("restart", ctypes.c_int32), ("gmres_prec", ctypes.c_int32), ("inner_tol", ctypes.c_double),
                ("residual", ctypes.c_int32), ("refine", ctypes.c_int32)]


class SolveReport(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("outer", ctypes.c_int32), ("inner", ctypes.c_int32),
                ("gmres_prec", ctypes.c_int32), ("bwd_err", ctypes.c_double), ("anorm_inf", ctypes.c_double),
                ("factor_ms", ctypes.c_double), ("solve_ms", ctypes.c_double), ("remedy", ctypes.c_int32),
                ("h2d_ms", ctypes.c_double), ("d2h_ms", ctypes.c_double), ("compute_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class BatchArgs(ctypes.Structure):
    _fields_ = [("n_systems", ctypes.c_int32), ("sizes", ctypes.POINTER(ctypes.c_int32)), ("tile", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("nrhs", ctypes.c_int32), ("ir_steps", ctypes.c_int32),
                ("seed", ctypes.c_uint32), ("alpha", ctypes.c_double), ("priority", ctypes.c_int32)]


class BatchReport(ctypes.Structure):
    _fields_ = [("run", Report), ("tasks", ctypes.c_int64), ("flops", ctypes.c_double)]


class ServeArgs(ctypes.Structure):
    _fields_ = [("n_requests", ctypes.c_int32), ("rate", ctypes.c_double), ("n_min", ctypes.c_int32), ("n_max", ctypes.c_int32),
                ("alpha", ctypes.c_double), ("seed", ctypes.c_uint32), ("followup_frac", ctypes.c_double),
                ("precision", ctypes.c_int32), ("ir_steps", ctypes.c_int32), ("nrhs", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("max_batch", ctypes.c_int32), ("hbm_budget_gb", ctypes.c_double), ("tol", ctypes.c_double),
                ("keep_results", ctypes.c_int32), ("admission", ctypes.c_int32)]


class ServeReport(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int32), ("factorisations", ctypes.c_int32), ("followups", ctypes.c_int32),
                ("followup_misses", ctypes.c_int32), ("evictions", ctypes.c_int32), ("launches", ctypes.c_int32),
                ("retries", ctypes.c_int32), ("unconverged", ctypes.c_int32), ("wall_s", ctypes.c_double),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("solves_per_s", ctypes.c_double), ("tflops", ctypes.c_double),
                ("worst_bwd_err", ctypes.c_double), ("peak_gb", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# Every symbol the public headers declare, with its ctypes signature.
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_STATUS = ctypes.c_int
SIGNATURES = {
    # include/ttg.h
    "ttg_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "ttg_last_cuda_error": (ctypes.c_char_p, []),
    "ttg_kernel_launches": (ctypes.c_int64, []),
    "ttg_team_item": (_STATUS, [ctypes.c_int32, ctypes.c_int32, _P, _P, _P, _P]),
    "ttg_create": (_STATUS, [ctypes.POINTER(_P), ctypes.POINTER(Opts)]),
    "ttg_destroy": (_STATUS, [_P]),
    "ttg_graph_upload": (_STATUS, [_P, ctypes.POINTER(GraphDesc)]),
    "ttg_launch": (_STATUS, [_P, _P]),
    "ttg_wait": (_STATUS, [_P, ctypes.POINTER(Report)]),
    "ttg_run": (_STATUS, [_P, _P, ctypes.POINTER(Report)]),
    "ttg_task_record": (_STATUS, [_P, _P, _P]),
    "ttg_trace": (_STATUS, [_P, _P, _P, _P]),
    "ttg_trace_busy": (_STATUS, [_P, _P]),
    "ttg_critical_path_priority": (_STATUS, [_P, _P]),
    "ttg_workers": (ctypes.c_int, [_P]),
    "ttg_set_workers": (_STATUS, [_P, _I32]),
    # include/ttg_serve.h
    "ttg_serve_tile": (_I32, [_I32]),
    "ttg_serve_create": (_STATUS, [ctypes.c_int, ctypes.POINTER(ServeArgs), ctypes.POINTER(_P)]),
    "ttg_serve_destroy": (None, [_P]),
    "ttg_serve_run": (_STATUS, [_P, ctypes.POINTER(ServeReport), _P]),
    "ttg_serve_request": (_STATUS, [_P, _I32, _P, _P, _P, _P, _P, _P, _P, _P]),
    "ttg_serve_get_x": (_STATUS, [_P, _I32, _P]),
    # include/ttg_batch.h
    "ttg_batch_create": (_STATUS, [_P, ctypes.POINTER(BatchArgs), ctypes.POINTER(_P)]),
    "ttg_batch_destroy": (None, [_P]),
    "ttg_batch_generate": (_STATUS, [_P, _P]),
    "ttg_batch_set_system": (_STATUS, [_P, _I32, _P, _P, _P]),
    "ttg_batch_run": (_STATUS, [_P, _P, ctypes.POINTER(BatchReport)]),
    "ttg_batch_get_x": (_STATUS, [_P, _I32, _P]),
    "ttg_batch_backward_errors": (_STATUS, [_P, _P, _P]),
    "ttg_batch_autotune": (_STATUS, [_P, ctypes.POINTER(BatchArgs), _P, _I32, _P, _I32, _I32, _P, _P,
                                     ctypes.POINTER(ctypes.c_double)]),
    "ttg_graph_generation": (ctypes.c_uint64, [_P]),
    "ttg_gen_gram_tiles": (_STATUS, [_P, _I32, _P, _I32, ctypes.c_double, ctypes.c_uint32, _P, _P]),
    "ttg_gen_uniform": (_STATUS, [_P, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32, _P, _P]),
    "ttg_gen_normal": (_STATUS, [_P, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32, _P, _P]),
    "ttg_tile_layout": (ctypes.c_int64, [_P, _I32, _P]),
    "ttg_measure_fp64_peak": (_STATUS, [_P, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "ttg_run_graph_noalloc": (_STATUS, [ctypes.c_int, ctypes.POINTER(GraphDesc), ctypes.c_int, ctypes.c_double, _P,
                                        ctypes.POINTER(Report)]),
    # include/ttg_apps.h
    "ttg_chol_plan_create": (_STATUS, [_P, ctypes.POINTER(CholArgs), ctypes.POINTER(_P)]),
    "ttg_chol_plan_destroy": (_STATUS, [_P]),
    "ttg_chol_plan_n": (_I32, [_P, _P]),
    "ttg_chol_plan_tasks": (_I32, [_P, ctypes.POINTER(ctypes.c_double)]),
    "ttg_chol_plan_generate": (_STATUS, [_P, _P]),
    "ttg_chol_plan_set_matrix": (_STATUS, [_P, _P, _P]),
    "ttg_chol_plan_restore": (_STATUS, [_P, _P]),
    "ttg_chol_plan_factor": (_STATUS, [_P, _P, ctypes.POINTER(Report)]),
    "ttg_chol_factor_host": (_STATUS, [_P, _P, _P, _P, ctypes.POINTER(Report)]),
    "ttg_chol_plan_get_factor": (_STATUS, [_P, _P]),
    "ttg_chol_factor_host_tiles": (_STATUS, [_P, _P, _P, _P, ctypes.POINTER(Report)]),
    "ttg_chol_plan_tile_elems": (ctypes.c_int64, [_P]),
    "ttg_chol_plan_copy_tiles": (_STATUS, [_P, _I32, _P]),
    "ttg_chol_plan_get_input": (_STATUS, [_P, _P]),
    "ttg_chol_plan_tiles": (_P, [_P, _P]),
    "ttg_chol_plan_dump_dag": (_STATUS, [_P, ctypes.c_char_p]),
    "ttg_chol_plan_kind_times": (_STATUS, [_P, _P, _P, _P, _P]),
    "ttg_chol_plan_trace_dump": (_STATUS, [_P, ctypes.c_char_p]),
    "ttg_chol_plan_write_log": (_STATUS, [_P, ctypes.c_char_p, ctypes.c_char_p]),
    "ttg_chol_plan_remedy": (ctypes.c_int32, [_P]),
    "ttg_chol_dag_dump": (_STATUS, [ctypes.POINTER(CholArgs), ctypes.c_char_p]),
    "ttg_gemm_dag_dump": (_STATUS, [ctypes.POINTER(GemmArgs), ctypes.c_char_p]),
    "ttg_chol_plan_solve": (_STATUS, [_P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveReport), _P]),
    "ttg_chol_posv": (_STATUS, [_P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveReport), _P]),
    "ttg_chol_posv_host": (_STATUS, [_P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveReport), _P]),
    "ttg_split_f64_f32": (_STATUS, [_P, ctypes.c_int64, _P, _P]),
    "ttg_sliced_matmul": (_STATUS, [_P, _I32, _P, _I32, _P, _P, _P, _I32, _P]),
    "ttg_chol_solve_host": (_STATUS, [_P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveReport), _P]),
    "ttg_gemm_plan_create": (_STATUS, [_P, ctypes.POINTER(GemmArgs), ctypes.POINTER(_P)]),
    "ttg_gemm_plan_destroy": (_STATUS, [_P]),
    "ttg_gemm_plan_tasks": (_I32, [_P, ctypes.POINTER(ctypes.c_double)]),
    "ttg_gemm_plan_run": (_STATUS, [_P, _P, ctypes.POINTER(Report)]),
    "ttg_gemm_host": (_STATUS, [_P, _P, _P, _P, _P, ctypes.POINTER(Report)]),
    "ttg_gemm_plan_get_C": (_STATUS, [_P, _P]),
    "ttg_gemm_plan_dump_dag": (_STATUS, [_P, ctypes.c_char_p]),
}

_lib = None


def lib():
    """The loaded libttg.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libttg.so is not built (run __graft_entry__.build()): %s" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def strerror(s):
    try:
        return lib().ttg_strerror(s).decode()
    except Exception:
        return "status %d" % s


def check(status, what):
    if status != TTG_OK:
        raise TTGError(status, what)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Context:
    """A device context (ttg_create)."""

    def fp64_peak(self, ms=200.0):
        """Measured FP64 FMA throughput (TFLOP/s) of the device."""
        v = ctypes.c_double()
        check(lib().ttg_measure_fp64_peak(self.h, ms, ctypes.byref(v)), "ttg_measure_fp64_peak")
        return v.value

    def __init__(self, device=0, workers=0, timeout_s=10.0, trace=False):
        self.h = ctypes.c_void_p()
        o = Opts(device, workers, timeout_s, 1 if trace else 0)
        check(lib().ttg_create(ctypes.byref(self.h), ctypes.byref(o)), "ttg_create")

    @property
    def workers(self):
        return lib().ttg_workers(self.h)

    def close(self):
        if self.h:
            lib().ttg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, ops, init_count, succ_ptr, succ_idx, priority=None, bind=None):
        """Upload a graph given as numpy arrays / a list of Op."""
        n = len(init_count)
        ops_arr = (Op * max(1, n))(*ops)
        ic = np.ascontiguousarray(init_count, dtype=np.int32)
        sp = np.ascontiguousarray(succ_ptr, dtype=np.int64)
        si = np.ascontiguousarray(succ_idx if len(succ_idx) else [0], dtype=np.int32)
        pr = None if priority is None else np.ascontiguousarray(priority, dtype=np.float64)
        bd = None if bind is None else np.ascontiguousarray(bind, dtype=np.int32)
        g = GraphDesc(n, ops_arr, ic.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                      pr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if pr is not None else None,
                      bd.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if bd is not None else None,
                      sp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), si.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        return lib().ttg_graph_upload(self.h, ctypes.byref(g))

    def run(self, stream=None):
        rep = Report()
        st = lib().ttg_run(self.h, stream, ctypes.byref(rep))
        return st, rep

    def task_record(self, n):
        runs = np.zeros(n, dtype=np.int32)
        cnt = np.zeros(n, dtype=np.int32)
        check(lib().ttg_task_record(self.h, _ptr(runs), _ptr(cnt)), "ttg_task_record")
        return runs, cnt

    def trace(self, n):
        s = np.zeros(n, dtype=np.int64)
        e = np.zeros(n, dtype=np.int64)
        w = np.zeros(n, dtype=np.int32)
        check(lib().ttg_trace(self.h, _ptr(s), _ptr(e), _ptr(w)), "ttg_trace")
        return s, e, w

    def trace_busy(self, n):
        b = np.zeros(n, dtype=np.int64)
        check(lib().ttg_trace_busy(self.h, _ptr(b)), "ttg_trace_busy")
        return b


def critical_path_priority(ops, succ_ptr, succ_idx):
    """Longest remaining path (estimated device µs) of every task of a graph
    (host computation, no device needed).  Returns (status, priorities)."""
    n = len(ops)
    ops_arr = (Op * max(1, n))(*ops)
    sp = np.ascontiguousarray(succ_ptr, dtype=np.int64)
    si = np.ascontiguousarray(succ_idx if len(succ_idx) else [0], dtype=np.int32)
    g = GraphDesc(n, ops_arr, None, None, None, sp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                  si.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    out = np.zeros(max(1, n), dtype=np.float64)
    st = lib().ttg_critical_path_priority(ctypes.byref(g), _ptr(out))
    return st, out[:n]


def dag_edges_from_lists(n, succ_lists):
    ptr = np.zeros(n + 1, dtype=np.int64)
    idx = []
    for t in range(n):
        idx.extend(succ_lists[t])
        ptr[t + 1] = len(idx)
    return ptr, np.array(idx, dtype=np.int32)


def chol_dag_dump(prefix, block_size, num_blocks, n_threads=4, kind=0, accumulate=False, upper_block_size=-1):
    """Capture the Cholesky task graph on the host (no GPU) and write its DAG record."""
    a = CholArgs(n_threads, 0, block_size, num_blocks, kind, 1 if accumulate else 0, upper_block_size, 0, 1.0, 0, PREC_F64, 0)
    check(lib().ttg_chol_dag_dump(ctypes.byref(a), prefix.encode()), "ttg_chol_dag_dump")


def gemm_dag_dump(prefix, matrix_size, block_size, n_threads=4):
    """Capture the block GEMM task graph on the host (no GPU) and write its DAG record."""
    a = GemmArgs(n_threads, 0, block_size, matrix_size, 1, 1)
    check(lib().ttg_gemm_dag_dump(ctypes.byref(a), prefix.encode()), "ttg_gemm_dag_dump")


class CholPlan:
    """A tiled Cholesky plan (ttg_chol_plan_*)."""

    def __init__(self, ctx, block_size, num_blocks, n_threads=8, kind=0, accumulate=False, upper_block_size=-1,
                 matrix=1, alpha=1.0, seed=0, precision=PREC_F64, mixed_kind=0, verb=0):
        self.ctx = ctx
        self.args = CholArgs(n_threads, verb, block_size, num_blocks, kind, 1 if accumulate else 0, upper_block_size,
                             matrix, alpha, seed, precision, mixed_kind)
        self.h = ctypes.c_void_p()
        check(lib().ttg_chol_plan_create(ctx.h, ctypes.byref(self.args), ctypes.byref(self.h)), "ttg_chol_plan_create")
        self.block_sizes = np.zeros(num_blocks, dtype=np.int32)
        self.N = lib().ttg_chol_plan_n(self.h, _ptr(self.block_sizes))

    def tasks(self):
        c = ctypes.c_double()
        n = lib().ttg_chol_plan_tasks(self.h, ctypes.byref(c))
        return n, c.value

    def factor(self, restore=True, stream=None):
        if restore:
            check(lib().ttg_chol_plan_restore(self.h, stream), "restore")
        rep = Report()
        st = lib().ttg_chol_plan_factor(self.h, stream, ctypes.byref(rep))
        return st, rep

    def set_matrix(self, A):
        A = np.asfortranarray(A, dtype=np.float64)
        check(lib().ttg_chol_plan_set_matrix(self.h, _ptr(A), None), "set_matrix")

    def factor_host(self, A, want_L=True):
        A = np.asfortranarray(A, dtype=np.float64)
        L = np.zeros((self.N, self.N), dtype=np.float64, order="F") if want_L else None
        rep = Report()
        st = lib().ttg_chol_factor_host(self.h, _ptr(A), _ptr(L), None, ctypes.byref(rep))
        return st, rep, L

    def tile_elems(self):
        return lib().ttg_chol_plan_tile_elems(self.h)

    def factor_host_tiles(self, h_in, h_out=None, stream=None):
        """End-to-end through host buffers in the packed lower-tile layout
        (numpy arrays, ideally pinned)."""
        rep = Report()
        def addr(x):
            return ctypes.c_void_p(x.ctypes.data if hasattr(x, "ctypes") else x) if x is not None else None
        st = lib().ttg_chol_factor_host_tiles(self.h, addr(h_in), addr(h_out), stream, ctypes.byref(rep))
        return st, rep

    def copy_tiles(self, which, h_dst):
        """Packed tiles to a host buffer (numpy array or raw address)."""
        addr = h_dst.ctypes.data if hasattr(h_dst, "ctypes") else h_dst
        check(lib().ttg_chol_plan_copy_tiles(self.h, which, ctypes.c_void_p(addr)), "copy_tiles")

    def factor_L(self):
        L = np.zeros((self.N, self.N), dtype=np.float64, order="F")
        check(lib().ttg_chol_plan_get_factor(self.h, _ptr(L)), "get_factor")
        return L

    def input_A(self):
        A = np.zeros((self.N, self.N), dtype=np.float64, order="F")
        check(lib().ttg_chol_plan_get_input(self.h, _ptr(A)), "get_input")
        return A

    def dump_dag(self, prefix):
        check(lib().ttg_chol_plan_dump_dag(self.h, prefix.encode()), "dump_dag")

    def solve_host(self, B, tiles=None, tol=1e-14, max_outer=10, restart=20, gmres_prec=0, inner_tol=0.0, factor=True,
                   residual=0, refine=0):
        """Factor (unless factor=False) and solve A X = B with host arrays
        (B: N×nrhs).  residual: 0 auto, 1 FP64 FMA, 2 sliced tensor-core
        products; refine: 0 classic steps then GMRES, 1 GMRES only.
        Returns (status, SolveReport, X)."""
        B = np.asfortranarray(B, dtype=np.float64)
        if B.ndim == 1:
            B = B.reshape(-1, 1, order="F")
        X = np.zeros_like(B, order="F")
        o = SolveOpts(B.shape[1], tol, max_outer, restart, gmres_prec, inner_tol, residual, refine)
        rep = SolveReport()
        if factor:
            st = lib().ttg_chol_posv_host(self.h, _ptr(tiles) if tiles is not None else None, _ptr(B), _ptr(X),
                                          ctypes.byref(o), ctypes.byref(rep), None)
        else:
            st = lib().ttg_chol_solve_host(self.h, _ptr(B), _ptr(X), ctypes.byref(o), ctypes.byref(rep), None)
        return st, rep, X

    def trace_dump(self, path):
        """Per-task timeline of the last run (context created with trace=True)."""
        check(lib().ttg_chol_plan_trace_dump(self.h, path.encode()), "ttg_chol_plan_trace_dump")

    def kind_times(self):
        v = [ctypes.c_double() for _ in range(4)]
        st = lib().ttg_chol_plan_kind_times(self.h, *[ctypes.byref(x) for x in v])
        return st, [x.value for x in v]

    def close(self):
        if self.h:
            lib().ttg_chol_plan_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GemmPlan:
    """A 2D block GEMM plan (ttg_gemm_plan_*)."""

    def __init__(self, ctx, matrix_size, block_size, n_threads=8, inputs=1, seed=1, verb=0):
        self.ctx = ctx
        self.N = matrix_size
        self.args = GemmArgs(n_threads, verb, block_size, matrix_size, inputs, seed)
        self.h = ctypes.c_void_p()
        check(lib().ttg_gemm_plan_create(ctx.h, ctypes.byref(self.args), ctypes.byref(self.h)), "ttg_gemm_plan_create")

    def tasks(self):
        c = ctypes.c_double()
        n = lib().ttg_gemm_plan_tasks(self.h, ctypes.byref(c))
        return n, c.value

    def run(self, stream=None):
        rep = Report()
        st = lib().ttg_gemm_plan_run(self.h, stream, ctypes.byref(rep))
        return st, rep

    def host(self, A, B, want_C=True):
        A = np.asfortranarray(A, dtype=np.float64)
        B = np.asfortranarray(B, dtype=np.float64)
        C = np.zeros((self.N, self.N), dtype=np.float64, order="F") if want_C else None
        rep = Report()
        st = lib().ttg_gemm_host(self.h, _ptr(A), _ptr(B), _ptr(C), None, ctypes.byref(rep))
        return st, rep, C

    def C(self):
        C = np.zeros((self.N, self.N), dtype=np.float64, order="F")
        check(lib().ttg_gemm_plan_get_C(self.h, _ptr(C)), "get_C")
        return C

    def dump_dag(self, prefix):
        check(lib().ttg_gemm_plan_dump_dag(self.h, prefix.encode()), "dump_dag")

    def close(self):
        if self.h:
            lib().ttg_gemm_plan_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent SPD factor-and-solve systems in one executor launch
    (include/ttg_batch.h).  sizes: N_i; precision PREC_F64, or PREC_MIXED
    (FP32 factor and ir_steps refinement rounds in the same launch)."""

    def __init__(self, ctx, sizes, tile, precision=PREC_F64, nrhs=1, ir_steps=2, seed=3, alpha=1.0, priority=0,
                 generate=True):
        self.ctx = ctx
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        self.nrhs = nrhs
        self.args = BatchArgs(len(self.sizes), self.sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), tile, precision,
                              nrhs, ir_steps, seed, alpha, priority)
        h = _P()
        check(lib().ttg_batch_create(ctx.h, ctypes.byref(self.args), ctypes.byref(h)), "ttg_batch_create")
        self.h = h
        if generate:
            check(lib().ttg_batch_generate(self.h, None), "ttg_batch_generate")

    def set_system(self, i, A=None, B=None):
        n = int(self.sizes[i])
        A = None if A is None else np.asfortranarray(A, dtype=np.float64)
        B = None if B is None else np.asfortranarray(np.asarray(B, dtype=np.float64).reshape(n, -1))
        check(lib().ttg_batch_set_system(self.h, i, _ptr(A), _ptr(B), None), "ttg_batch_set_system")

    def run(self, stream=None):
        rep = BatchReport()
        st = lib().ttg_batch_run(self.h, stream, ctypes.byref(rep))
        return st, rep

    def x(self, i):
        out = np.zeros((int(self.sizes[i]), self.nrhs), order="F")
        check(lib().ttg_batch_get_x(self.h, i, _ptr(out)), "ttg_batch_get_x")
        return out

    def backward_errors(self):
        out = np.zeros(len(self.sizes))
        check(lib().ttg_batch_backward_errors(self.h, _ptr(out), None), "ttg_batch_backward_errors")
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().ttg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_autotune(ctx, sizes, tiles, workers, precision=PREC_F64, nrhs=1, ir_steps=2, seed=3, alpha=1.0, max_sample=400):
    """Fastest (tile, workers) for a batch of these sizes; returns (tile, workers, ms per system)."""
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    a = BatchArgs(len(sizes), sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 0, precision, nrhs, ir_steps, seed,
                  alpha, 0)
    tl = np.ascontiguousarray(tiles, dtype=np.int32)
    wk = np.ascontiguousarray(workers, dtype=np.int32)
    bt, bw, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
    check(lib().ttg_batch_autotune(ctx.h, ctypes.byref(a), _ptr(tl), len(tl), _ptr(wk), len(wk), max_sample,
                                   ctypes.byref(bt), ctypes.byref(bw), ctypes.byref(ms)), "ttg_batch_autotune")
    return bt.value, bw.value, ms.value


class Serve:
    """The request loop of include/ttg_serve.h (a Poisson stream of
    factor-and-solve and follow-up requests over `lanes` executors).
    admission 0: each lane takes the waiting requests as its next launch;
    1 (mixed precision): open lanes — a persistent executor per lane takes a
    request's tasks while it runs."""

    def __init__(self, n_requests, rate, n_min=64, n_max=8192, alpha=1e-4, seed=2, followup_frac=0.3,
                 precision=PREC_MIXED, ir_steps=4, nrhs=1, lanes=2, max_batch=16, hbm_budget_gb=180.0, tol=1e-14,
                 keep_results=False, device=0, admission=0):
        self.args = ServeArgs(n_requests, rate, n_min, n_max, alpha, seed, followup_frac, precision, ir_steps, nrhs, lanes,
                              max_batch, hbm_budget_gb, tol, 1 if keep_results else 0, admission)
        self.nrhs = nrhs
        h = _P()
        check(lib().ttg_serve_create(device, ctypes.byref(self.args), ctypes.byref(h)), "ttg_serve_create")
        self.h = h

    def run(self):
        rep = ServeReport()
        lat = np.zeros(self.args.n_requests)
        st = lib().ttg_serve_run(self.h, ctypes.byref(rep), _ptr(lat))
        return st, rep, lat

    def request(self, i):
        n, tile, fo, ir = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        sa, sb = ctypes.c_uint32(), ctypes.c_uint32()
        arr, be = ctypes.c_double(), ctypes.c_double()
        check(lib().ttg_serve_request(self.h, i, ctypes.byref(n), ctypes.byref(tile), ctypes.byref(sa), ctypes.byref(sb),
                                      ctypes.byref(arr), ctypes.byref(fo), ctypes.byref(be), ctypes.byref(ir)), "ttg_serve_request")
        return {"n": n.value, "tile": tile.value, "seed_a": sa.value, "seed_b": sb.value, "arrival_s": arr.value,
                "followup_of": fo.value, "bwd_err": be.value, "ir_steps": ir.value}

    def x(self, i):
        out = np.zeros((self.request(i)["n"], self.nrhs), order="F")
        check(lib().ttg_serve_get_x(self.h, i, _ptr(out)), "ttg_serve_get_x")
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().ttg_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

