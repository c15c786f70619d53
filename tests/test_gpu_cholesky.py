"""Tiled Cholesky on the GPU executor against the oracle: the input is
bit-identical, the DAG (tasks, indegrees, promises, edges, runs) equals the
reference runtime's, and the FP64 factor agrees to ‖LLᵀ−A‖/‖A‖ ≤ 1e-13."""
import os

import numpy as np
import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-13  # ‖LLᵀ−A‖_F / ‖A‖_F and ‖L−L_oracle‖_F / ‖L_oracle‖_F, FP64


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("b,nb,alpha,seed", [(32, 8, 1.0, 0), (64, 5, 1e-4, 2), (128, 16, 1.0, 0)])
def test_fp64_factor_matches_oracle(ctx, b, nb, alpha, seed):
    p = t.CholPlan(ctx, b, nb, n_threads=8, kind=2, matrix=1, alpha=alpha, seed=seed)
    st, rep = p.factor()
    assert st == t.TTG_OK, t.strerror(st)
    assert rep.tasks_run == rep.tasks_total and rep.bad_runs == 0
    A = p.input_A()
    r = orc.cholesky(block_size=b, num_blocks=nb, n_threads=8, kind=2, matrix=1, alpha=alpha, seed=seed, want_A=True)
    assert np.array_equal(A, r["A"])  # the device generator is bit-identical
    L = p.factor_L()
    assert rel(L @ L.T, A) <= TOL
    assert rel(L, r["L"]) <= TOL
    p.close()


def test_cfg1_n2048_tile128(ctx):
    """N = 2048, tile 128 (16×16 tiles, 816 tasks), A = G·Gᵀ/N + I, seed 0."""
    p = t.CholPlan(ctx, 128, 16, n_threads=8, kind=0, matrix=1, alpha=1.0, seed=0)
    n_tasks, _ = p.tasks()
    assert n_tasks == 816
    st, rep = p.factor()
    assert st == t.TTG_OK and rep.tasks_run == 816
    A = p.input_A()
    L = p.factor_L()
    assert rel(L @ L.T, A) <= TOL
    p.close()


@pytest.mark.parametrize("kind,acc", [(0, 0), (0, 1), (2, 0), (2, 1)])
def test_device_dag_equals_reference_runtime(ctx, tmp_path, kind, acc):
    p = t.CholPlan(ctx, 4, 16, n_threads=4, kind=kind, accumulate=bool(acc), matrix=0)
    st, rep = p.factor()
    assert st == t.TTG_OK
    pre = str(tmp_path / "d")
    p.dump_dag(pre)
    # Runs in the record are the DEVICE's per-task run counts.
    assert orc.read_dag(pre) == orc.read_dag(os.path.join(GOLDEN, "dag_chol_nb16_k%d_acc%d" % (kind, acc)))
    p.close()


@pytest.mark.parametrize("b,nb,upper,acc,kind", [(5, 10, -1, False, 0), (5, 10, 7, False, 3), (12, 9, 20, True, 1),
                                                 (33, 7, 50, True, 2), (1, 6, -1, False, 0)])
def test_uneven_blocks_and_accumulate(ctx, b, nb, upper, acc, kind):
    p = t.CholPlan(ctx, b, nb, n_threads=3, kind=kind, accumulate=acc, upper_block_size=upper, matrix=0)
    st, rep = p.factor()
    assert st == t.TTG_OK
    r = orc.cholesky(block_size=b, num_blocks=nb, n_threads=3, kind=kind, accumulate=acc, upper_block_size=upper, matrix=0,
                     want_A=True)
    assert list(p.block_sizes) == list(orc.block_sizes(b, nb, upper))
    L = p.factor_L()
    assert rel(L @ L.T, r["A"]) <= TOL
    assert rel(L, r["L"]) <= TOL
    p.close()


def test_host_path_equals_resident_path(ctx):
    p = t.CholPlan(ctx, 64, 6, matrix=1, alpha=1.0, seed=0)
    st, _ = p.factor()
    L1 = p.factor_L()
    A = p.input_A()
    st, rep, L2 = p.factor_host(A)
    assert st == t.TTG_OK
    assert np.array_equal(L1, L2)
    p.close()


@pytest.mark.parametrize("mk,b", [(1, 64), (2, 128)])
def test_host_path_equals_resident_path_mixed(ctx, mk, b):
    """A mixed plan's host path factors the host matrix (written as the plan's
    input) and returns the mixed factor: the resident path's bits.  FP32
    updates (mixed_kind 1) take any tile; split-BF16 tensor-core updates
    (mixed_kind 2) need tiles that are a multiple of 128."""
    p = t.CholPlan(ctx, b, 6, matrix=1, alpha=1.0, seed=0, precision=t.PREC_MIXED, mixed_kind=mk)
    st, _ = p.factor()
    assert st == t.TTG_OK
    L1 = p.factor_L()
    A = p.input_A()
    st, rep, L2 = p.factor_host(A)
    assert st == t.TTG_OK
    assert np.array_equal(L1, L2)
    assert np.linalg.norm(L2 @ L2.T - A) / np.linalg.norm(A) < 1e-5
    p.close()


def test_repeated_factorisations_are_identical(ctx):
    p = t.CholPlan(ctx, 96, 7, kind=2, matrix=1, alpha=1e-4, seed=2)
    outs = []
    for _ in range(3):
        st, _ = p.factor()
        assert st == t.TTG_OK
        outs.append(p.factor_L())
    # Each tile's updates run in the DAG's fixed k order: same bits every run.
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])
    p.close()


@pytest.mark.parametrize("prec,mk", [(None, 0), ("mixed", 1), ("mixed", 0)])
def test_critical_path_priorities_same_factor(ctx, tmp_path, prec, mk):
    """Priority kind 4 (longest remaining path) changes the order, not the DAG or the bits."""
    kw = dict(precision=t.PREC_MIXED, mixed_kind=mk) if prec else {}
    outs, dags = [], []
    for kind in (2, 4):
        p = t.CholPlan(ctx, 128, 6, kind=kind, matrix=1, alpha=1.0, seed=2, **kw)
        st, _ = p.factor()
        assert st == t.TTG_OK
        outs.append(p.factor_L())
        p.dump_dag(str(tmp_path / ("k%d" % kind)))
        dags.append((tmp_path / ("k%d.tasks.csv" % kind)).read_text() + (tmp_path / ("k%d.edges.csv" % kind)).read_text())
        p.close()
    assert np.array_equal(outs[0], outs[1])
    assert dags[0] == dags[1]


def test_not_positive_definite_is_reported(ctx):
    p = t.CholPlan(ctx, 16, 4, matrix=1, alpha=-1.0, seed=0)
    st, rep = p.factor()
    assert st == t.TTG_ENOTPD and rep.info >= 1
    p.close()


@pytest.mark.parametrize("mk,b,upper", [(2, 64, -1), (0, 96, -1), (2, 128, 200), (3, 64, -1), (4, 128, -1)])
def test_rejected_mixed_plan_allocates_nothing(ctx, mk, b, upper):
    """Tensor-core updates need uniform tiles that are a multiple of 128, and
    mixed_kind is 0 to 3: other requests return TTG_EINVAL and leave the
    device's free memory where it was."""
    import torch
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        with pytest.raises(t.TTGError) as e:
            t.CholPlan(ctx, b, 6, matrix=1, alpha=1.0, seed=0, precision=t.PREC_MIXED, mixed_kind=mk, upper_block_size=upper)
        assert e.value.status == t.TTG_EINVAL
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0


def test_plans_release_their_memory(ctx):
    """Creating and destroying FP64, mixed and GEMM plans returns the device
    memory they took."""
    import torch
    for _ in range(2):  # the first round sets up lazily created context buffers
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(0)
        p = t.CholPlan(ctx, 128, 8, matrix=1, alpha=1.0, seed=0)
        q = t.CholPlan(ctx, 128, 8, matrix=1, alpha=1.0, seed=0, precision=t.PREC_MIXED, mixed_kind=2)
        g = t.GemmPlan(ctx, 512, 128)
        p.close()
        q.close()
        g.close()
        free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
