"""The persistent executor through the C ABI: random DAGs (the reference's
graph.randomdag), the 8-task graph.mini, bound tasks, failure reporting, and
each FP64 tile kernel against numpy."""
import ctypes

import numpy as np
import pytest

import tasktorrent_gb300 as t

pytestmark = pytest.mark.gpu


def nop_graph(n, succ):
    ops = [t.Op(kind=t.OP_NOP) for _ in range(n)]
    indeg = np.zeros(n, dtype=np.int32)
    for s in succ:
        for d in s:
            indeg[d] += 1
    ptr, idx = t.dag_edges_from_lists(n, succ)
    return ops, indeg, ptr, idx


def random_dag(n, p, rng):
    # Strictly lower-triangular random edges j -> i (j < i), then a random
    # relabelling, as graph.randomdag does (tests/shared/tests.cpp:294-358).
    perm = rng.permutation(n)
    mask = np.tril(rng.random((n, n)) < p, k=-1)
    succ = [[] for _ in range(n)]
    ii, jj = np.nonzero(mask)
    for i, j in zip(ii, jj):
        succ[perm[j]].append(int(perm[i]))
    return succ


@pytest.mark.parametrize("n", [1, 3, 7, 30, 200, 3000])
@pytest.mark.parametrize("p", [0.0, 0.01, 0.2, 0.5])
def test_random_dag_each_task_once(ctx, n, p):
    if n * n * p > 2e6:
        pytest.skip("too many edges")
    rng = np.random.default_rng(2019 + n)
    succ = random_dag(n, p, rng)
    ops, indeg, ptr, idx = nop_graph(n, succ)
    prio = rng.random(n)
    t.check(ctx.upload(ops, indeg, ptr, idx, priority=prio), "upload")
    st, rep = ctx.run()
    assert st == t.TTG_OK, t.strerror(st)
    runs, cnt = ctx.task_record(n)
    assert (runs == 1).all() and (cnt == 0).all()
    assert rep.tasks_run == n and rep.bad_runs == 0 and rep.tasks_pending == 0
    # Order: every task started after all its predecessors ended.
    s, e, w = ctx.trace(n)
    src = np.repeat(np.arange(n), [len(x) for x in succ])
    dst = np.array([b for x in succ for b in x], dtype=np.int64)
    if len(dst):
        assert (s[dst] >= e[src]).all()


def test_graph_mini(ctx):
    # tests/shared/tests.cpp:130-183: indegrees {1,1,1,2,1,3,1,1}, seeds 0 and 7.
    out = [[1, 2], [3], [3, 5], [4, 6], [5], [], [], [5]]
    indegree = np.array([1, 1, 1, 2, 1, 3, 1, 1], dtype=np.int32)
    init = indegree.copy()
    init[0] -= 1
    init[7] -= 1
    ptr, idx = t.dag_edges_from_lists(8, out)
    ops = [t.Op(kind=t.OP_NOP) for _ in range(8)]
    t.check(ctx.upload(ops, init, ptr, idx, priority=np.arange(8.0)), "upload")
    for _ in range(3):  # re-launch: counters and queues are reset each time
        st, rep = ctx.run()
        assert st == t.TTG_OK and rep.tasks_run == 8


def test_bound_tasks_run_on_their_worker(ctx):
    W = ctx.workers
    n = 4 * W
    succ = [[] for _ in range(n)]
    for i in range(n - 1):
        if i % 3:
            succ[i].append(i + 1)
    ops, indeg, ptr, idx = nop_graph(n, succ)
    bind = np.array([(i * 7) % (2 * W) if i % 2 else -1 for i in range(n)], dtype=np.int32)
    t.check(ctx.upload(ops, indeg, ptr, idx, bind=bind), "upload")
    st, rep = ctx.run()
    assert st == t.TTG_OK and rep.tasks_run == n
    s, e, w = ctx.trace(n)
    for i in range(n):
        if bind[i] >= 0:
            assert w[i] == bind[i] % W


def test_overcount_is_reported(ctx):
    # Task 2 receives two promises but declares one.
    ops, indeg, ptr, idx = nop_graph(3, [[2], [2], []])
    indeg[2] = 1
    t.check(ctx.upload(ops, indeg, ptr, idx), "upload")
    st, rep = ctx.run()
    assert st == t.TTG_EOVERCOUNT


def test_underrun_runs_what_can_run(ctx):
    # Task 2 declares three promises but receives two: it never runs, the
    # others do (the reference never runs it either), and the run says so.
    ops, indeg, ptr, idx = nop_graph(4, [[2], [2], [], []])
    indeg[2] = 3
    t.check(ctx.upload(ops, indeg, ptr, idx), "upload")
    st, rep = ctx.run()
    assert st == t.TTG_EUNDERRUN
    runs, cnt = ctx.task_record(4)
    assert list(runs) == [1, 1, 0, 1] and cnt[2] == 1


def test_timeout_returns_and_context_stays_usable():
    """Idle workers give up after the no-progress limit while one long tile
    task runs; the kernel returns TTG_ETIMEOUT (no trap) and the next run on
    the same context succeeds."""
    import torch
    c = t.Context(device=0, timeout_s=0.02)
    n = 1536
    A = torch.rand(n, n, dtype=torch.float64, device="cuda")
    B = torch.rand(n, n, dtype=torch.float64, device="cuda")
    C = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    op = t.Op(kind=t.OP_GEMM_NN, m=n, n=n, k=n, lda=n, ldb=n, ldc=n, alpha=1.0, beta=0.0, a=A.data_ptr(), b=B.data_ptr(),
              c=C.data_ptr())
    t.check(c.upload([op], np.zeros(1, np.int32), np.zeros(2, np.int64), np.zeros(0, np.int32)), "upload")
    st, rep = c.run()
    assert st == t.TTG_ETIMEOUT
    ops, indeg, ptr, idx = nop_graph(5, [[1], [2], [3], [4], []])
    t.check(c.upload(ops, indeg, ptr, idx), "upload")
    st, rep = c.run()
    assert st == t.TTG_OK and rep.tasks_run == 5
    c.close()


def _colmajor(a):
    """Device copy of numpy array `a` stored column-major; returns (tensor, ptr)."""
    import torch
    tt = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # row-major of aᵀ == column-major of a
    return tt, tt.data_ptr()


def _back(tt, shape):
    return tt.cpu().numpy().T.reshape(shape)


def run_single(ctx, op):
    t.check(ctx.upload([op], np.zeros(1, np.int32), np.zeros(2, np.int64), np.zeros(0, np.int32)), "upload")
    st, rep = ctx.run()
    return st, rep


@pytest.mark.parametrize("parts", [0, 1, 3])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (17, 33, 5), (128, 128, 128), (200, 131, 257), (512, 512, 512)])
def test_gemm_kernels(ctx, m, n, k, parts):
    import torch
    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((m, k))
    Bt = rng.standard_normal((n, k))
    Bn = rng.standard_normal((k, n))
    C0 = rng.standard_normal((m, n))
    for kind, B, ref in ((t.OP_GEMM_NT, Bt, A @ Bt.T), (t.OP_GEMM_NN, Bn, A @ Bn)):
        dA, pA = _colmajor(A)
        dB, pB = _colmajor(B)
        dC, pC = _colmajor(C0)
        torch.cuda.synchronize()
        op = t.Op(kind=kind, m=m, n=n, k=k, lda=m, ldb=B.shape[0], ldc=m, parts=parts, alpha=-1.0, beta=1.0, a=pA, b=pB, c=pC)
        st, _ = run_single(ctx, op)
        assert st == t.TTG_OK
        got = _back(dC, (m, n))
        want = C0 - ref
        assert np.abs(got - want).max() <= 1e-13 * max(1.0, np.abs(want).max()) * k


@pytest.mark.parametrize("parts", [0, 2])
@pytest.mark.parametrize("n,k", [(1, 3), (40, 17), (128, 64), (300, 301), (512, 512)])
def test_syrk_kernel_lower_only(ctx, n, k, parts):
    import torch
    rng = np.random.default_rng(n * 7 + k)
    A = rng.standard_normal((n, k))
    C0 = rng.standard_normal((n, n))
    dA, pA = _colmajor(A)
    dC, pC = _colmajor(C0)
    torch.cuda.synchronize()
    op = t.Op(kind=t.OP_SYRK_LN, m=n, n=n, k=k, lda=n, ldc=n, parts=parts, alpha=-1.0, beta=1.0, a=pA, c=pC)
    assert run_single(ctx, op)[0] == t.TTG_OK
    got = _back(dC, (n, n))
    want = C0 - A @ A.T
    low = np.tril(np.ones((n, n), bool))
    assert np.abs(got[low] - want[low]).max() <= 1e-12 * k
    assert np.array_equal(got[~low], C0[~low])  # upper triangle untouched


@pytest.mark.parametrize("n", [1, 31, 32, 33, 100, 128, 256, 512])
def test_potrf_kernel(ctx, n):
    import torch
    rng = np.random.default_rng(n)
    G = rng.standard_normal((n, n))
    A = G @ G.T / n + np.eye(n)
    dA, pA = _colmajor(A)
    torch.cuda.synchronize()
    op = t.Op(kind=t.OP_POTRF_L, m=n, n=n, ldc=n, c=pA)
    st, rep = run_single(ctx, op)
    assert st == t.TTG_OK
    got = np.tril(_back(dA, (n, n)))
    L = np.linalg.cholesky(A)
    assert np.linalg.norm(got - L) <= 1e-13 * np.linalg.norm(L)
    assert np.linalg.norm(got @ got.T - A) <= 1e-14 * n * np.linalg.norm(A)


@pytest.mark.parametrize("n", [128, 300, 512, 1000])
@pytest.mark.parametrize("parts", [2, 5, 16, 64])
def test_potrf_team_matches_one_block(ctx, n, parts):
    """A POTRF shared by a team of blocks gives the single-block factor bit for bit."""
    import torch
    rng = np.random.default_rng(n + parts)
    G = rng.standard_normal((n, n))
    A = G @ G.T / n + np.eye(n)
    out = []
    for p in (1, parts):
        dA, pA = _colmajor(A)
        torch.cuda.synchronize()
        st, rep = run_single(ctx, t.Op(kind=t.OP_POTRF_L, m=n, n=n, ldc=n, parts=p, c=pA))
        assert st == t.TTG_OK
        out.append(_back(dA, (n, n)))
    assert np.array_equal(np.tril(out[0]), np.tril(out[1]))
    L = np.linalg.cholesky(A)
    assert np.linalg.norm(np.tril(out[1]) - L) <= 1e-13 * np.linalg.norm(L)


@pytest.mark.parametrize("parts", [0, 1, 4])
def test_empty_potrf_releases_its_successor(ctx, parts):
    """A 0×0 diagonal tile (ragged tilings can produce one) still completes."""
    ops = [t.Op(kind=t.OP_POTRF_L, m=0, n=0, ldc=1, parts=parts), t.Op(kind=t.OP_NOP)]
    ptr, idx = t.dag_edges_from_lists(2, [[1], []])
    t.check(ctx.upload(ops, np.array([0, 1], np.int32), ptr, idx), "upload")
    st, rep = ctx.run()
    assert st == t.TTG_OK and rep.tasks_run == 2


def test_potrf_team_not_positive_definite(ctx):
    import torch
    n = 300
    A = np.eye(n) * 2.0
    A[201, 201] = -1.0
    dA, pA = _colmajor(A)
    torch.cuda.synchronize()
    st, rep = run_single(ctx, t.Op(kind=t.OP_POTRF_L, m=n, n=n, ldc=n, parts=8, c=pA))
    assert st == t.TTG_ENOTPD and rep.info == 202 and rep.error_task == 0


def test_potrf_not_positive_definite(ctx):
    import torch
    n = 70
    A = np.eye(n)
    A[45, 45] = -1.0
    dA, pA = _colmajor(A)
    torch.cuda.synchronize()
    st, rep = run_single(ctx, t.Op(kind=t.OP_POTRF_L, m=n, n=n, ldc=n, c=pA))
    assert st == t.TTG_ENOTPD and rep.info == 46 and rep.error_task == 0


@pytest.mark.parametrize("parts", [0, 1, 5])
@pytest.mark.parametrize("m,n,alpha", [(1, 1, 1.0), (50, 33, 1.0), (300, 128, 2.0), (512, 512, 1.0)])
def test_trsm_kernel(ctx, m, n, alpha, parts):
    import torch
    rng = np.random.default_rng(m + 3 * n)
    G = rng.standard_normal((n, n))
    L = np.linalg.cholesky(G @ G.T / n + np.eye(n))
    B = rng.standard_normal((m, n))
    dL, pL = _colmajor(L)
    dB, pB = _colmajor(B)
    torch.cuda.synchronize()
    op = t.Op(kind=t.OP_TRSM_RLTN, m=m, n=n, lda=n, ldc=m, parts=parts, alpha=alpha, a=pL, c=pB)
    assert run_single(ctx, op)[0] == t.TTG_OK
    got = _back(dB, (m, n))
    want = np.linalg.solve(L, (alpha * B).T).T
    assert np.linalg.norm(got @ L.T - alpha * B) <= 1e-13 * np.linalg.norm(B) * max(1, alpha)
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)


def test_geadd_kernel(ctx):
    import torch
    rng = np.random.default_rng(5)
    A = rng.standard_normal((77, 45))
    C = rng.standard_normal((77, 45))
    dA, pA = _colmajor(A)
    dC, pC = _colmajor(C)
    torch.cuda.synchronize()
    op = t.Op(kind=t.OP_GEADD, m=77, n=45, lda=77, ldc=77, parts=3, alpha=2.0, beta=1.0, a=pA, c=pC)
    assert run_single(ctx, op)[0] == t.TTG_OK
    assert np.allclose(_back(dC, (77, 45)), 2 * A + C, rtol=0, atol=1e-15)
