"""Mixed Cholesky with BF16 trailing updates on tcgen05 tensor cores (TMA
operands, TMEM accumulators): factor accuracy at BF16 level, identical task
graph, and GMRES-IR to FP64 backward error."""
import os

import numpy as np
import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BWD = 1e-14


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def bwd_err(A, X, B):
    R = B - A @ X
    return np.max(np.abs(R).max(axis=0) / (np.abs(A).sum(axis=1).max() * np.abs(X).max(axis=0)))


@pytest.mark.parametrize("b,nb", [(128, 2), (256, 2), (128, 5), (512, 4)])
def test_bf16_factor_accuracy(ctx, b, nb):
    p = t.CholPlan(ctx, b, nb, kind=2, matrix=1, alpha=1.0, seed=0, precision=t.PREC_MIXED, mixed_kind=0)
    st, rep = p.factor()
    assert st == t.TTG_OK, t.strerror(st)
    assert rep.tasks_run == rep.tasks_total and rep.bad_runs == 0
    A = p.input_A()
    L = p.factor_L()
    e = rel(L @ L.T, A)
    # BF16 operands (8-bit mantissa), FP32 accumulation: ~1e-3 relative.
    assert 1e-6 < e < 2e-2, e
    # Compare with the FP32-update factor: same graph, lower-precision products.
    q = t.CholPlan(ctx, b, nb, kind=2, matrix=1, alpha=1.0, seed=0, precision=t.PREC_MIXED, mixed_kind=1)
    st, _ = q.factor()
    assert st == t.TTG_OK
    assert rel(L, q.factor_L()) < 2e-2
    p.close()
    q.close()


def test_remedy_chain_on_ill_conditioned_input(ctx):
    """alpha = 1e-8: the BF16 factor loses definiteness; the plan retries
    (FP32 updates, then shifted factors) and still returns a usable factor."""
    p = t.CholPlan(ctx, 128, 8, kind=2, matrix=1, alpha=1e-8, seed=2, precision=t.PREC_MIXED, mixed_kind=0)
    st, rep = p.factor()
    assert st == t.TTG_OK
    assert t.lib().ttg_chol_plan_remedy(p.h) in (0, 1, 2, 3, 4)
    L = p.factor_L()
    assert np.isfinite(L).all()
    p.close()


def test_bf16_repeatable(ctx):
    p = t.CholPlan(ctx, 256, 4, kind=2, matrix=1, alpha=1.0, seed=1, precision=t.PREC_MIXED, mixed_kind=0)
    Ls = []
    for _ in range(2):
        st, _ = p.factor()
        assert st == t.TTG_OK
        Ls.append(p.factor_L())
    assert np.array_equal(Ls[0], Ls[1])  # fixed k order per tile: same bits
    p.close()


@pytest.mark.parametrize("alpha,max_outer", [(1.0, 10), (1e-4, 15), (1e-8, 30)])
def test_bf16_gmres_ir_to_fp64_backward_error(ctx, alpha, max_outer):
    p = t.CholPlan(ctx, 128, 8, kind=2, matrix=1, alpha=alpha, seed=2, precision=t.PREC_MIXED, mixed_kind=0)
    A = p.input_A()
    B = orc.normals(0, p.N * 16, 9, 1).reshape(p.N, 16, order="F")
    st, rep, X = p.solve_host(B, tol=BWD, max_outer=max_outer, restart=30)
    assert st == t.TTG_OK, rep.as_dict()
    # alpha = 1: BF16 updates as they are; smaller alpha may need the
    # remedies (FP32 updates, diagonal shifts) — the result must not depend on it.
    if alpha == 1.0:
        assert rep.remedy == 0
    assert rep.bwd_err <= BWD and bwd_err(A, X, B) <= 2 * BWD
    Xref = np.linalg.solve(A, B)
    assert rel(X, Xref) <= max(1e-12, 1e-15 * np.linalg.cond(A) * 100)
    p.close()


@pytest.mark.parametrize("b,nb", [(128, 3), (256, 2), (512, 3)])
def test_split_bf16_factor_is_fp32_accurate(ctx, b, nb):
    """Split-BF16 updates (three BF16 slices, six tensor-core products) give a
    factor as accurate as FP32 updates, far better than plain BF16."""
    errs = {}
    for mk in (0, 1, 2):
        p = t.CholPlan(ctx, b, nb, kind=2, matrix=1, alpha=1.0, seed=4, precision=t.PREC_MIXED, mixed_kind=mk)
        st, rep = p.factor()
        assert st == t.TTG_OK, t.strerror(st)
        assert rep.tasks_run == rep.tasks_total and rep.bad_runs == 0
        A = p.input_A()
        errs[mk] = rel(p.factor_L() @ p.factor_L().T, A)
        p.close()
    assert errs[2] < 1e-5, errs
    assert errs[2] < errs[0] / 30, errs
    # Measured 1.0×, 1.1×, 1.6× the FP32-update error for tiles 128, 256, 512;
    # adding the small slice products onto the hi·hi accumulator (rather
    # than into their own) costs enough accuracy to show here.
    assert errs[2] < 2 * errs[1], errs


def test_split_bf16_refines_an_ill_conditioned_system(ctx):
    """alpha = 1e-4: plain BF16 loses definiteness; split BF16 (first attempt
    of mixed_kind 2) factors it and GMRES-IR reaches FP64 backward error."""
    p = t.CholPlan(ctx, 128, 8, kind=2, matrix=1, alpha=1e-4, seed=2, precision=t.PREC_MIXED, mixed_kind=2)
    A = p.input_A()
    B = orc.normals(0, p.N * 4, 9, 1).reshape(p.N, 4, order="F")
    st, rep, X = p.solve_host(B, tol=BWD, max_outer=10, restart=30)
    assert st == t.TTG_OK, rep.as_dict()
    assert rep.remedy == 4
    assert rep.bwd_err <= BWD and bwd_err(A, X, B) <= 2 * BWD
    p.close()


def test_split_bf16_preconditions_an_ill_conditioned_system(ctx):
    """alpha = 1e-8 (cond ~ 1e9): FP64 Krylov GMRES-IR preconditioned by the
    split-BF16 factor converges in few iterations (10 measured at N = 2048) —
    a guard on the factor's accuracy, which sets the preconditioner quality."""
    p = t.CholPlan(ctx, 256, 8, kind=2, matrix=1, alpha=1e-8, seed=2, precision=t.PREC_MIXED, mixed_kind=2)
    A = p.input_A()
    B = orc.normals(0, p.N * 4, 11, 1).reshape(p.N, 4, order="F")
    st, rep, X = p.solve_host(B, tol=BWD, max_outer=12, restart=30, gmres_prec=64)
    assert st == t.TTG_OK, rep.as_dict()
    assert rep.remedy == 4
    assert rep.inner <= 14, rep.as_dict()
    assert rep.bwd_err <= BWD and bwd_err(A, X, B) <= 2 * BWD
    p.close()


@pytest.mark.parametrize("b,nb", [(128, 3), (256, 2), (512, 3)])
def test_split_fp16_factor_accuracy(ctx, b, nb):
    """Split-FP16 updates (two FP16 slices, the remainder scaled by 2^11;
    three tensor-core products) give a factor near FP32 accuracy, far better
    than plain BF16, from the same task graph."""
    errs, dags = {}, {}
    for mk in (0, 1, 3):
        p = t.CholPlan(ctx, b, nb, kind=2, matrix=1, alpha=1.0, seed=4, precision=t.PREC_MIXED, mixed_kind=mk)
        st, rep = p.factor()
        assert st == t.TTG_OK, t.strerror(st)
        assert rep.tasks_run == rep.tasks_total and rep.bad_runs == 0
        A = p.input_A()
        errs[mk] = rel(p.factor_L() @ p.factor_L().T, A)
        p.close()
    assert errs[3] < 1e-5, errs
    assert errs[3] < errs[0] / 30, errs
    assert errs[3] < 8 * errs[1], errs


@pytest.mark.parametrize("alpha", [1e-4, 1e-8])
def test_split_fp16_refines_to_fp64_backward_error(ctx, alpha):
    """The split-FP16 factor keeps definiteness at alpha = 1e-4 (no remedy:
    remedy 5) and the refinement reaches FP64 backward error; at 1e-8 its
    first refinement step gains less than 10x, so the plan factors again
    with split-BF16 updates (remedy 4) and converges from there."""
    p = t.CholPlan(ctx, 128, 8, kind=2, matrix=1, alpha=alpha, seed=2, precision=t.PREC_MIXED, mixed_kind=3)
    A = p.input_A()
    B = orc.normals(0, p.N * 4, 9, 1).reshape(p.N, 4, order="F")
    st, rep, X = p.solve_host(B, tol=BWD, max_outer=30, restart=30)
    assert st == t.TTG_OK, rep.as_dict()
    assert rep.remedy == (5 if alpha == 1e-4 else 4), rep.as_dict()
    assert rep.bwd_err <= BWD and bwd_err(A, X, B) <= 2 * BWD
    p.close()
