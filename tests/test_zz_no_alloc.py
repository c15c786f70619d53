"""ttg_run_graph_noalloc: the executor for callers that cannot allocate device
memory (a service whose pool owns the free HBM, an operator hosted by a
framework that only allows its own allocator, a caller that cannot afford an
allocation's device-wide synchronisation).  Its scratch is one fixed device
array inside libttg.so.

The test runs one tiled-Cholesky task graph through the regular entry point
(ttg_graph_upload + ttg_run, which allocates) and through the no-alloc entry
point twice in a row, and compares the factors with the tolerance of the
other Cholesky tests.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import tasktorrent_gb300 as t

pytestmark = pytest.mark.gpu
TOL = 1e-13  # relative Frobenius, FP64, as the other Cholesky tests


def cholesky_graph(base, b, nb):
    """Right-looking tiled Cholesky task graph (potrf, trsm, syrk/gemm chained
    over k) on packed lower tiles of b×b doubles at device address `base`."""
    off = {}
    o = 0
    for j in range(nb):
        for i in range(j, nb):
            off[(i, j)] = o
            o += b * b
    tile = lambda i, j: base + 8 * off[(i, j)]
    ids, ops = {}, []

    def task(key, op):
        ids[key] = len(ops)
        ops.append(op)

    for j in range(nb):
        task(("P", j), t.Op(kind=t.OP_POTRF_L, m=b, n=b, ldc=b, c=tile(j, j)))
        for i in range(j + 1, nb):
            task(("T", i, j), t.Op(kind=t.OP_TRSM_RLTN, m=b, n=b, lda=b, ldc=b, alpha=1.0, a=tile(j, j), c=tile(i, j)))
    for j in range(nb):
        for i in range(j, nb):
            for k in range(j):
                if i == j:
                    op = t.Op(kind=t.OP_SYRK_LN, m=b, n=b, k=b, lda=b, ldc=b, alpha=-1.0, beta=1.0, a=tile(i, k), c=tile(i, i))
                else:
                    op = t.Op(kind=t.OP_GEMM_NT, m=b, n=b, k=b, lda=b, ldb=b, ldc=b, alpha=-1.0, beta=1.0, a=tile(i, k),
                              b=tile(j, k), c=tile(i, j))
                task(("G", k, i, j), op)
    succ = [[] for _ in ops]
    for key, tid in ids.items():
        if key[0] == "P":
            j = key[1]
            succ[tid] = [ids[("T", i, j)] for i in range(j + 1, nb)]
        elif key[0] == "T":
            i, j = key[1], key[2]
            succ[tid] = [ids[("G", j, i, k)] for k in range(j + 1, i)] + [ids[("G", j, k, i)] for k in range(i, nb)]
        else:
            k, i, j = key[1:]
            succ[tid] = [ids[("G", k + 1, i, j)]] if k < j - 1 else [ids[("P", i)] if i == j else ids[("T", i, j)]]
    indeg = np.zeros(len(ops), dtype=np.int32)
    for s in succ:
        for d in s:
            indeg[d] += 1
    ptr, idx = t.dag_edges_from_lists(len(ops), succ)
    return ops, indeg, ptr, idx, off


def to_dense(tiles, off, b, nb):
    N = b * nb
    L = np.zeros((N, N))
    for (i, j), o in off.items():
        L[i * b:(i + 1) * b, j * b:(j + 1) * b] = tiles[o:o + b * b].reshape(b, b, order="F")
    return np.tril(L)


def graph_desc(ops, indeg, ptr, idx, prio=None):
    n = len(ops)
    keep = [(t.Op * n)(*ops), np.ascontiguousarray(indeg, np.int32), np.ascontiguousarray(ptr, np.int64),
            np.ascontiguousarray(idx if len(idx) else [0], np.int32),
            None if prio is None else np.ascontiguousarray(prio, np.float64)]
    g = t.GraphDesc(n, keep[0], keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                    None if prio is None else keep[4].ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None,
                    keep[2].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                    keep[3].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return g, keep


def kind2_priorities(b, nb):
    """Priorities of the tasks of cholesky_graph in 2d_cholesky's --kind 2
    form: potrf 9(nb-j)-1, trsm 9(nb-j)-2, gemm 9nb-9j-2 (fewer distinct
    values than the executor's 128 levels)."""
    pr = []
    for j in range(nb):
        pr.append(9 * (nb - j) - 1)
        pr += [9 * (nb - j) - 2] * (nb - 1 - j)
    for j in range(nb):
        for i in range(j, nb):
            pr += [9 * nb - 9 * j - 2] * j
    return np.array(pr, np.float64)


@pytest.mark.parametrize("with_priorities", [False, True])
def test_noalloc_matches_regular_entry_point(ctx, with_priorities):
    import torch
    b, nb = 64, 6
    N = b * nb
    rng = np.random.default_rng(11)
    G = rng.standard_normal((N, N))
    A = G @ G.T / N + np.eye(N)
    # Packed lower tiles of A (column-major inside each tile).
    probe = cholesky_graph(0, b, nb)[4]
    packed = np.zeros(b * b * len(probe))
    for (i, j), o in probe.items():
        packed[o:o + b * b] = A[i * b:(i + 1) * b, j * b:(j + 1) * b].reshape(-1, order="F")
    ref_dev = torch.from_numpy(packed.copy()).cuda()
    na_dev = torch.from_numpy(packed.copy()).cuda()
    torch.cuda.synchronize()

    # Regular entry point (allocates the graph, counters and queues).
    ops, indeg, ptr, idx, off = cholesky_graph(ref_dev.data_ptr(), b, nb)
    t.check(ctx.upload(ops, indeg, ptr, idx), "upload")
    st, rep = ctx.run()
    assert st == t.TTG_OK and rep.tasks_run == len(ops)
    L_ref = to_dense(ref_dev.cpu().numpy(), off, b, nb)
    assert np.linalg.norm(L_ref @ L_ref.T - A) <= TOL * np.linalg.norm(A)

    # No-alloc entry point, two calls in a row on the same input.
    ops, indeg, ptr, idx, off = cholesky_graph(na_dev.data_ptr(), b, nb)
    prio = kind2_priorities(b, nb) if with_priorities else None
    assert prio is None or len(prio) == len(ops)
    g, keep = graph_desc(ops, indeg, ptr, idx, prio)
    for call in range(2):
        na_dev.copy_(torch.from_numpy(packed))
        torch.cuda.synchronize()
        rep = t.Report()
        st = t.lib().ttg_run_graph_noalloc(0, ctypes.byref(g), 0, 20.0, None, ctypes.byref(rep))
        assert st == t.TTG_OK, t.strerror(st)
        assert rep.tasks_run == len(ops) and rep.bad_runs == 0 and rep.tasks_pending == 0
        L = to_dense(na_dev.cpu().numpy(), off, b, nb)
        assert np.linalg.norm(L - L_ref) <= TOL * np.linalg.norm(L_ref), "call %d" % call
        assert np.linalg.norm(L @ L.T - A) <= TOL * np.linalg.norm(A)


def test_noalloc_rejects_graphs_beyond_its_limits():
    n = 16385  # TTG_NOALLOC_MAX_TASKS + 1
    ops = [t.Op(kind=t.OP_NOP) for _ in range(n)]
    g, keep = graph_desc(ops, np.zeros(n, np.int32), np.zeros(n + 1, np.int64), np.zeros(0, np.int32))
    rep = t.Report()
    assert t.lib().ttg_run_graph_noalloc(0, ctypes.byref(g), 0, 5.0, None, ctypes.byref(rep)) == t.TTG_EINVAL


def test_noalloc_rejects_mixed_precision_ops():
    """Only FP64 tile operations: a mixed-precision op is refused before
    anything reaches the device."""
    op = t.Op(kind=t.OP_POTRF_L, prec=t.PREC_MIXED, m=64, n=64, ldc=64, c=0)
    g, keep = graph_desc([op], np.zeros(1, np.int32), np.zeros(2, np.int64), np.zeros(0, np.int32))
    rep = t.Report()
    assert t.lib().ttg_run_graph_noalloc(0, ctypes.byref(g), 0, 5.0, None, ctypes.byref(rep)) == t.TTG_EINVAL
