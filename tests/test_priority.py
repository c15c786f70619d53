"""Critical-path priorities (host computation on the graph, no device): the
longest remaining path in estimated device time."""
import numpy as np

import tasktorrent_gb300 as t


def _ops(kinds, n=256):
    return [t.Op(kind=k, prec=t.PREC_F64, m=n, n=n, k=n) for k in kinds]


def _csr(n, edges):
    succ = [[] for _ in range(n)]
    for a, b in edges:
        succ[a].append(b)
    ptr = np.zeros(n + 1, np.int64)
    idx = []
    for v in range(n):
        idx += succ[v]
        ptr[v + 1] = len(idx)
    return ptr, np.array(idx, np.int32)


def test_chain_decreases_along_the_path():
    ops = _ops([t.OP_POTRF_L, t.OP_TRSM_RLTN, t.OP_SYRK_LN, t.OP_POTRF_L])
    ptr, idx = _csr(4, [(0, 1), (1, 2), (2, 3)])
    st, pr = t.critical_path_priority(ops, ptr, idx)
    assert st == t.TTG_OK
    assert pr[0] > pr[1] > pr[2] > pr[3] > 0


def test_longer_branch_wins():
    # 0 -> 1 (cheap no-op) -> 3 ; 0 -> 2 (GEMM) -> 3: task 2 is on the critical path.
    ops = _ops([t.OP_NOP, t.OP_NOP, t.OP_GEMM_NT, t.OP_POTRF_L])
    ptr, idx = _csr(4, [(0, 1), (0, 2), (1, 3), (2, 3)])
    st, pr = t.critical_path_priority(ops, ptr, idx)
    assert st == t.TTG_OK
    assert pr[2] > pr[1]
    # A task's value is its own cost plus its heaviest successor's: both no-ops cost the same.
    assert np.isclose(pr[0] - pr[2], pr[1] - pr[3])


def test_cycle_is_rejected():
    ops = _ops([t.OP_NOP, t.OP_NOP])
    ptr, idx = _csr(2, [(0, 1), (1, 0)])
    st, _ = t.critical_path_priority(ops, ptr, idx)
    assert st == t.TTG_EINVAL


def test_bad_edge_is_rejected():
    ops = _ops([t.OP_NOP])
    st, _ = t.critical_path_priority(ops, np.array([0, 1], np.int64), np.array([5], np.int32))
    assert st == t.TTG_EINVAL
