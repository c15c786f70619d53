"""The C-ABI library loads and exports every function the public headers
declare; the drop-in's captured task graphs equal the reference runtime's.
CPU only: no call here touches a GPU."""
import os
import re
import subprocess

import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h") or h == "ttg_philox.h":  # header-only generator, no library symbols
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        # Prototypes only (header-only inline helpers such as ttg_philox.h
        # define their bodies in the header).
        for m in re.finditer(r"\b(ttg_\w+)\s*\([^;{}]*\)\s*;", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_function():
    names = declared_functions()
    assert len(names) > 30
    out = subprocess.run(["nm", "-D", "--defined-only", t.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = sorted(names - exported)
    assert not missing, missing
    lib = t.lib()
    for n in names:
        assert getattr(lib, n) is not None
    # The Python bindings cover every declared function.
    assert names <= set(t.SIGNATURES), sorted(names - set(t.SIGNATURES))


def test_strerror_without_gpu():
    assert t.strerror(t.TTG_OK) == "ok"
    assert "positive definite" in t.strerror(t.TTG_ENOTPD)


def test_serve_rejects_bad_arguments_before_any_device_call():
    """ttg_serve_create checks its arguments first: each bad field gives
    TTG_EINVAL with no GPU present (a device call would give TTG_ECUDA)."""
    import ctypes
    good = dict(n_requests=10, rate=100.0, n_min=64, n_max=512, alpha=1e-4, seed=2, followup_frac=0.3,
                precision=t.PREC_MIXED, ir_steps=3, nrhs=1, lanes=2, max_batch=4, hbm_budget_gb=1.0, tol=1e-14,
                keep_results=0, admission=0)
    bad = [dict(admission=2), dict(admission=-1), dict(admission=1, precision=t.PREC_F64), dict(lanes=0),
           dict(nrhs=17), dict(n_max=32), dict(rate=0.0), dict(precision=7)]
    for b in bad:
        args = t.ServeArgs(**dict(good, **b))
        h = ctypes.c_void_p()
        assert t.lib().ttg_serve_create(0, ctypes.byref(args), ctypes.byref(h)) == t.TTG_EINVAL, b
        assert not h.value


@pytest.mark.parametrize("kind,acc", [(0, 0), (0, 1), (2, 0), (2, 1)])
def test_captured_cholesky_dag_equals_reference(tmp_path, kind, acc):
    pre = str(tmp_path / "c")
    t.chol_dag_dump(pre, 4, 16, n_threads=4, kind=kind, accumulate=bool(acc))
    assert orc.read_dag(pre) == orc.read_dag(os.path.join(GOLDEN, "dag_chol_nb16_k%d_acc%d" % (kind, acc)))


def test_captured_gemm_dag_equals_reference(tmp_path):
    pre = str(tmp_path / "g")
    t.gemm_dag_dump(pre, 64, 4, n_threads=4)
    assert orc.read_dag(pre) == orc.read_dag(os.path.join(GOLDEN, "dag_gemm_nb16"))


@pytest.mark.parametrize("nb,nt,kind,acc,upper", [(1, 1, 0, 0, -1), (2, 3, 1, 1, -1), (9, 5, 3, 0, 7), (12, 8, 2, 1, 9)])
def test_captured_cholesky_dag_equals_oracle(tmp_path, nb, nt, kind, acc, upper):
    pre_t, pre_o = str(tmp_path / "t"), str(tmp_path / "o")
    t.chol_dag_dump(pre_t, 5, nb, n_threads=nt, kind=kind, accumulate=bool(acc), upper_block_size=upper)
    orc.cholesky(block_size=5, num_blocks=nb, n_threads=nt, kind=kind, accumulate=bool(acc), upper_block_size=upper,
                 matrix=0, want_L=False, dag_prefix=pre_o)
    assert orc.read_dag(pre_t) == orc.read_dag(pre_o)


def read_prio(prefix):
    out = {}
    with open(prefix + ".prio.csv") as f:
        next(f)
        for line in f:
            n, v = line.strip().split(",")
            out[n] = float(v)
    return out


def task_coords(name):
    parts = name.split("_")
    return parts[0], [int(x) for x in parts[1:]]


@pytest.mark.parametrize("kind", [2, 6])
def test_captured_priorities_follow_the_kind(tmp_path, kind):
    """--kind 2 is the reference's formula (2d_cholesky.cpp: potrf 9(nb-j)-1,
    trsm and gemm 9(nb-j)-2 by the target column j); kind 6 (extension) puts
    the tasks of the tiles within two of the diagonal above every other task,
    by column, and leaves the rest as kind 2."""
    nb = 12
    pre = str(tmp_path / "p")
    t.chol_dag_dump(pre, 4, nb, n_threads=4, kind=kind)
    prio = read_prio(pre)
    assert len(prio) == nb + nb * (nb - 1) // 2 + sum(j * (nb - j) for j in range(nb))
    chain, bulk = [], []
    for name, v in prio.items():
        kd, c = task_coords(name)
        if kd == "POTRF":
            i = j = c[0]
        elif kd == "TRSM":
            i, j = c
        else:  # GEMM_k_i_j
            i, j = c[1], c[2]
        k2 = 9 * (nb - j) - (1 if kd == "POTRF" else 2)
        if kind == 2:
            assert v == k2, name
        elif i <= j + 2:
            assert v == 9 * nb + 9 * (nb - j), name
            chain.append(v)
        else:
            assert v == 9 * (nb - j) - 2, name
            bulk.append(v)
    if kind == 6:
        assert min(chain) > max(bulk)
        assert len(set(chain)) + len(set(bulk)) <= 2 * nb  # fits the executor's 128 levels up to 64 tile columns


@pytest.mark.parametrize("N,b", [(8, 8), (24, 8), (40, 4)])
def test_captured_gemm_dag_equals_oracle(tmp_path, N, b):
    pre_t, pre_o = str(tmp_path / "t"), str(tmp_path / "o")
    t.gemm_dag_dump(pre_t, N, b, n_threads=3)
    orc.gemm(N, b, n_threads=3, want_C=False, dag_prefix=pre_o)
    assert orc.read_dag(pre_t) == orc.read_dag(pre_o)


def test_cli_help_and_bad_args():
    for prog in ("2d_cholesky", "2d_gemm"):
        exe = os.path.join(t.BIN_DIR, prog)
        r = subprocess.run([exe, "--help"], capture_output=True, text=True)
        assert r.returncode == 0 and "--block_size" in r.stdout
        r = subprocess.run([exe, "--nprows=2"], capture_output=True, text=True)
        assert r.returncode == 2
        r = subprocess.run([exe, "--no_such_flag=1"], capture_output=True, text=True)
        assert r.returncode == 2


def _noalloc_desc(ops, indeg, ptr, idx):
    import ctypes
    import numpy as np
    n = len(ops)
    keep = [(t.Op * n)(*ops), np.ascontiguousarray(indeg, np.int32), np.ascontiguousarray(ptr, np.int64),
            np.ascontiguousarray(idx if len(idx) else [0], np.int32)]
    g = t.GraphDesc(n, keep[0], keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), None, None,
                    keep[2].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                    keep[3].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return g, keep


def test_noalloc_rejects_bad_graphs_before_any_device_call():
    """ttg_run_graph_noalloc validates the whole graph on the host first:
    every malformed case returns TTG_EINVAL with no GPU present."""
    import ctypes
    import numpy as np
    nop = t.Op(kind=t.OP_NOP)
    cases = [
        ([nop] * 16385, np.zeros(16385), np.zeros(16386), []),                     # beyond the task limit
        ([t.Op(kind=t.OP_POTRF_L, prec=t.PREC_MIXED, m=64, n=64, ldc=64)], [0], [0, 0], []),  # not FP64
        ([nop, nop], [0, 1], [0, 1, 1], [2]),                                       # successor out of range
        ([nop, nop], [0, -1], [0, 0, 0], []),                                       # negative counter
        ([nop, nop], [0, 1], [1, 1, 1], [1]),                                       # offsets not from 0
        ([t.Op(kind=99)], [0], [0, 0], []),                                         # unknown kind
    ]
    for ops, indeg, ptr, idx in cases:
        g, keep = _noalloc_desc(ops, indeg, ptr, idx)
        rep = t.Report()
        assert t.lib().ttg_run_graph_noalloc(0, ctypes.byref(g), 0, 5.0, None, ctypes.byref(rep)) == t.TTG_EINVAL


def _sweep_items(nb, bs, backward):
    """Decode every item of one sweep direction as the TMA sweep kernel does:
    (kind, step, strip) with kind 0 = diagonal strip D, 1 = Z strip of the
    next row, 2 = bulk update of strip g; and each item's inputs, from the
    kernel's wait conditions (folded form)."""
    sp = [0]
    for b in bs:
        sp.append(sp[-1] + (b + 63) // 64)
    row = (lambda s: nb - 1 - s) if backward else (lambda s: s)
    strips = lambda r: sp[r + 1] - sp[r]
    items = []
    for s in range(nb):
        i = row(s)
        items += [(0, s, sp[i] + u) for u in range(strips(i))]
        if s + 1 < nb:
            nx = row(s + 1)
            items += [(1, s, sp[nx] + u) for u in range(strips(nx))]
        if backward:  # rows i-2 … 0, last strip first
            bulk = range(sp[i - 1] - 1, -1, -1) if i >= 1 else range(0)
        else:  # rows i+2 … nb-1
            bulk = range(sp[min(i + 2, nb)], sp[nb])
        items += [(2, s, g) for g in bulk]
    index = {it: n for n, it in enumerate(items)}

    def inputs(it):
        kind, s, g = it
        if kind == 0:
            if s == 0:
                return []
            i, p = row(s), row(s - 1)
            return [index[(1, s - 1, h)] for h in range(sp[i], sp[i + 1])] + \
                   [index[(0, s - 1, h)] for h in range(sp[p], sp[p + 1])]
        if kind == 1:
            return [index[(2, s - 1, g)]] if s > 0 else []
        i = row(s)
        return [index[(0, s, h)] for h in range(sp[i], sp[i + 1])] + ([index[(2, s - 1, g)]] if s > 0 else [])
    return items, inputs


@pytest.mark.parametrize("bs", [[512], [512] * 2, [512] * 3, [512] * 7, [128] * 16, [64, 512, 200, 128, 1, 300]])
def test_sweep_claim_order_is_a_topological_order(bs):
    """The TMA sweeps' claim order (ttg_solve.cu) is a permutation of each
    direction's items in which every item follows all the items it waits
    for, so blocks claiming in that order never wait on an unclaimed item."""
    import ctypes
    import numpy as np
    f = t.lib().ttg_internal_sweep_order
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    nb = len(bs)
    b = np.asarray(bs, np.int32)
    n = f(nb, b.ctypes.data, None, 0)
    out = np.zeros(n, np.int32)
    assert f(nb, b.ctypes.data, out.ctypes.data, n) == n
    off = 0
    for backward in (0, 1):
        items, inputs = _sweep_items(nb, bs, backward)
        order = out[off: off + len(items)]
        off += len(items)
        assert sorted(order.tolist()) == list(range(len(items)))
        pos = np.empty(len(items), np.int64)
        pos[order] = np.arange(len(items))
        for k, it in enumerate(items):
            assert all(pos[d] < pos[k] for d in inputs(it)), (backward, it)
    assert off == n


@pytest.mark.parametrize("factored", [0, 1])
@pytest.mark.parametrize("tc", [0, 1])
def test_open_lane_bounds_cover_every_request_graph(factored, tc):
    """An open serving lane reserves room for a request from a closed-form
    bound before it builds the request's graph (ttg_serve.cu); the graph it
    then appends (the system's tasks and its last task) stays within the
    bound's tasks, 8 edges and 32 executor parts per bounded task, for every
    request size the serving tile rule produces and up to 12 refinement
    rounds (3, doubled twice on retries)."""
    import ctypes
    import numpy as np
    f = t.lib().ttg_internal_open_request_graph
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int32] * 7 + [ctypes.c_void_p]
    out = np.zeros(5, np.int64)
    sizes = sorted(set([64, 65, 100, 127, 128, 129, 255, 256, 257, 300, 511, 512, 700, 1000, 1023, 1024, 1500, 2047, 2048,
                        2049, 2304, 3000, 4096, 5000, 8191, 8192]))
    for N in sizes:
        tile = t.lib().ttg_serve_tile(N)
        for ir in (0, 3, 6, 12):
            for nrhs in (1, 16):
                assert f(N, tile, nrhs, ir, 1, factored, tc, out.ctypes.data) == t.TTG_OK
                bound, tasks, edges, parts, nb = out.tolist()
                assert tasks <= bound and edges <= 8 * bound and parts <= 32 * bound, (N, tile, ir, nrhs, out.tolist())
