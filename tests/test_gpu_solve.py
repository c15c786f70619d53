"""Solves with a Cholesky plan's factor: FP64 direct, and the mixed path
(low-precision factor + GMRES-IR, convergence on FP64 residuals) to backward error
≤ 1e-14; forward errors against the FP64 oracle solution."""
import numpy as np
import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
BWD = 1e-14  # ‖b − A x‖∞ / (‖A‖∞ ‖x‖∞), per column


def bwd_err(A, X, B):
    R = B - A @ X
    return np.max(np.abs(R).max(axis=0) / (np.abs(A).sum(axis=1).max() * np.abs(X).max(axis=0)))


def rhs(N, nrhs, seed=9):
    return orc.normals(0, N * nrhs, seed, 1).reshape(N, nrhs, order="F")


@pytest.mark.parametrize("b,nb,alpha,nrhs", [(64, 8, 1.0, 1), (128, 8, 1e-4, 16), (96, 10, 1e-8, 4)])
def test_fp64_direct_solve(ctx, b, nb, alpha, nrhs):
    p = t.CholPlan(ctx, b, nb, kind=2, matrix=1, alpha=alpha, seed=2)
    A = p.input_A()
    B = rhs(p.N, nrhs)
    st, rep, X = p.solve_host(B)
    assert st == t.TTG_OK, t.strerror(st)
    assert rep.bwd_err <= 1e-15 * 10 and bwd_err(A, X, B) <= 1e-15 * 10
    Xref = np.linalg.solve(A, B)
    kappa = np.linalg.cond(A)
    assert np.linalg.norm(X - Xref) / np.linalg.norm(Xref) <= 1e-15 * kappa * 100
    p.close()


@pytest.mark.parametrize("b,nb,upper,nrhs", [(100, 7, 150, 5), (70, 9, 139, 16), (200, 3, 260, 2)])
def test_fp64_direct_solve_ragged_tiles(ctx, b, nb, upper, nrhs):
    """Irregular tile sizes: strips that end mid-tile, tiles narrower than a strip."""
    p = t.CholPlan(ctx, b, nb, kind=2, matrix=1, alpha=1e-2, seed=3, upper_block_size=upper)
    A = p.input_A()
    B = rhs(p.N, nrhs, seed=4)
    st, rep, X = p.solve_host(B)
    assert st == t.TTG_OK, t.strerror(st)
    assert rep.bwd_err <= 1e-14 and bwd_err(A, X, B) <= 1e-14
    p.close()


def test_mixed_ragged_tiles_fp32_updates(ctx):
    p = t.CholPlan(ctx, 90, 8, kind=2, matrix=1, alpha=1e-4, seed=5, upper_block_size=170, precision=t.PREC_MIXED,
                   mixed_kind=1)
    A = p.input_A()
    B = rhs(p.N, 7, seed=6)
    st, rep, X = p.solve_host(B)
    assert st == t.TTG_OK, t.strerror(st)
    assert bwd_err(A, X, B) <= BWD
    p.close()


def test_mixed_factor_is_fp32_accurate(ctx):
    p = t.CholPlan(ctx, 64, 8, kind=2, matrix=1, alpha=1.0, seed=0, precision=t.PREC_MIXED, mixed_kind=1)
    st, rep = p.factor()
    assert st == t.TTG_OK
    A = p.input_A()
    L = p.factor_L()
    e = np.linalg.norm(L @ L.T - A) / np.linalg.norm(A)
    assert 1e-9 < e < 1e-5  # FP32 trailing updates: FP32-level, not FP64-level
    p.close()


@pytest.mark.parametrize("nrhs", [1, 2, 3, 16])
def test_mixed_small_nrhs(ctx, nrhs):
    p = t.CholPlan(ctx, 64, 6, matrix=1, alpha=1e-4, seed=3, precision=t.PREC_MIXED, mixed_kind=1)
    A = p.input_A()
    B = rhs(p.N, nrhs, seed=nrhs)
    st, rep, X = p.solve_host(B)
    assert st == t.TTG_OK, rep.as_dict()
    assert np.isfinite(X).all()
    assert bwd_err(A, X, B) <= 2 * BWD, rep.as_dict()
    p.close()


@pytest.mark.parametrize("alpha", [1.0, 1e-4, 1e-8])
@pytest.mark.parametrize("gprec", [0, 64])
def test_mixed_gmres_ir_reaches_fp64_backward_error(ctx, alpha, gprec):
    p = t.CholPlan(ctx, 128, 8, kind=2, matrix=1, alpha=alpha, seed=2, precision=t.PREC_MIXED, mixed_kind=1)
    A = p.input_A()
    B = rhs(p.N, 16)
    st, rep, X = p.solve_host(B, tol=BWD, gmres_prec=gprec, max_outer=12)
    assert st == t.TTG_OK, (t.strerror(st), rep.as_dict())
    assert rep.bwd_err <= BWD
    assert bwd_err(A, X, B) <= 2 * BWD
    Xref = np.linalg.solve(A, B)
    kappa = np.linalg.cond(A)
    assert np.linalg.norm(X - Xref) / np.linalg.norm(Xref) <= max(1e-12, 1e-15 * kappa * 100)
    p.close()


def test_follow_up_rhs_reuse_factor(ctx):
    p = t.CholPlan(ctx, 64, 6, matrix=1, alpha=1e-4, seed=3, precision=t.PREC_MIXED, mixed_kind=1)
    A = p.input_A()
    B1 = rhs(p.N, 2, seed=1)
    st, rep1, X1 = p.solve_host(B1)
    assert st == t.TTG_OK
    assert bwd_err(A, X1, B1) <= 2 * BWD
    B2 = rhs(p.N, 3, seed=2)
    st, rep2, X2 = p.solve_host(B2, factor=False)  # resident factor
    assert st == t.TTG_OK and rep2.factor_ms == 0.0
    assert bwd_err(A, X2, B2) <= 2 * BWD
    p.close()


@pytest.mark.parametrize("nrhs", [3, 16])
def test_device_pointer_solve_matches_host_path(ctx, nrhs):
    """ttg_chol_plan_solve on device buffers owned by the caller (here torch
    tensors) gives the host path's solution."""
    import ctypes
    import torch
    p = t.CholPlan(ctx, 64, 6, matrix=1, alpha=1e-4, seed=3, precision=t.PREC_MIXED, mixed_kind=1)
    A = p.input_A()
    B = rhs(p.N, nrhs, seed=5)
    st, rep, Xh = p.solve_host(B)
    assert st == t.TTG_OK
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dX = torch.zeros_like(dB)
    torch.cuda.synchronize()
    o = t.SolveOpts(nrhs, BWD, 10, 20, 0, 0.0)
    r = t.SolveReport()
    st = t.lib().ttg_chol_plan_solve(p.h, ctypes.c_void_p(dB.data_ptr()), ctypes.c_void_p(dX.data_ptr()), ctypes.byref(o),
                                     ctypes.byref(r), None)
    torch.cuda.synchronize()
    assert st == t.TTG_OK, r.as_dict()
    Xd = np.asfortranarray(dX.cpu().numpy().T)
    assert np.isfinite(Xd).all()
    assert bwd_err(A, Xd, B) <= 2 * BWD
    assert np.linalg.norm(Xd - Xh) <= 1e-10 * np.linalg.norm(Xh)
    p.close()


@pytest.mark.parametrize("mk", [1, 2])
def test_mixed_factor_reads_the_input(ctx, mk):
    """A mixed factorisation converts the plan's input itself (no restore of
    the FP64 working tiles, which are the diagonal POTRF's scratch): two
    factorisations in a row, without a restore, give the same factor bits,
    and a matrix set afterwards is the one factored."""
    p = t.CholPlan(ctx, 128, 6, kind=2, matrix=1, alpha=1.0, seed=4, precision=t.PREC_MIXED, mixed_kind=mk)
    st, _ = p.factor(restore=False)
    assert st == t.TTG_OK
    L1 = p.factor_L()
    st, _ = p.factor(restore=False)
    assert st == t.TTG_OK
    assert np.array_equal(p.factor_L(), L1)
    A2 = p.input_A() + 2.0 * np.eye(p.N)
    p.set_matrix(A2)
    st, _ = p.factor(restore=False)
    assert st == t.TTG_OK
    L2 = p.factor_L()
    assert np.linalg.norm(L2 @ L2.T - A2) / np.linalg.norm(A2) < 1e-5
    p.close()


@pytest.mark.parametrize("tol", [1e-9, 1e-11])
def test_reported_backward_error_is_fp64_at_a_loose_tolerance(ctx, tol):
    """Early refinement residuals may be double-float estimates; the one that
    decides convergence, and the reported backward error, are FP64: the report
    matches the backward error recomputed on the host."""
    p = t.CholPlan(ctx, 256, 8, kind=2, matrix=1, alpha=1e-4, seed=2, precision=t.PREC_MIXED, mixed_kind=2)
    A = p.input_A()
    B = rhs(p.N, 16, seed=7)
    st, rep, X = p.solve_host(B, tol=tol, max_outer=12)
    assert st == t.TTG_OK, rep.as_dict()
    host = bwd_err(A, X, B)
    assert rep.bwd_err <= tol and host <= 2 * tol
    assert abs(rep.bwd_err - host) <= 1e-3 * host + 1e-17, (rep.bwd_err, host)
    p.close()


@pytest.mark.parametrize("mk", [1, 2])
def test_host_tiles_replace_the_input(ctx, mk):
    """ttg_chol_posv_host with new host tiles: the plan factors and solves the
    new matrix (its dense copies are rebuilt), and later calls without tiles
    keep it as the resident input."""
    kw = dict(kind=2, matrix=1, alpha=1e-4, precision=t.PREC_MIXED, mixed_kind=mk)
    p = t.CholPlan(ctx, 128, 6, seed=2, **kw)
    q = t.CholPlan(ctx, 128, 6, seed=5, **kw)
    A1, A2 = p.input_A(), q.input_A()
    assert not np.array_equal(A1, A2)
    tiles2 = np.empty(q.tile_elems(), dtype=np.float64)
    q.copy_tiles(1, tiles2)
    B = rhs(p.N, 4, seed=11)
    st, rep, X1 = p.solve_host(B)
    assert st == t.TTG_OK and bwd_err(A1, X1, B) <= 2 * BWD
    st, rep, X2 = p.solve_host(B, tiles=tiles2)
    assert st == t.TTG_OK, rep.as_dict()
    assert bwd_err(A2, X2, B) <= 2 * BWD and rep.bwd_err <= BWD
    st, rep, X3 = p.solve_host(B)
    assert st == t.TTG_OK and bwd_err(A2, X3, B) <= 2 * BWD
    assert np.array_equal(X3, X2)
    p.close()
    q.close()


@pytest.mark.parametrize("alpha", [1.0, 1e-4, 1e-8])
def test_classic_steps_then_gmres(ctx, alpha):
    """refine 0 (classic steps x += M⁻¹r while each gains 10×, then GMRES) and
    refine 1 (GMRES from the start) both reach the FP64 backward error; a
    well-conditioned matrix needs no GMRES iteration at all."""
    p = t.CholPlan(ctx, 128, 6, matrix=1, alpha=alpha, seed=2, precision=t.PREC_MIXED, mixed_kind=2)
    A = p.input_A()
    B = np.random.default_rng(4).standard_normal((p.N, 8))
    reps = {}
    for refine in (0, 1):
        st, rep, X = p.solve_host(B, tol=BWD, max_outer=30, restart=30, refine=refine)
        assert st == t.TTG_OK, (refine, rep.as_dict())
        R = B - A @ X
        bwd = np.max(np.abs(R).max(axis=0) / (np.abs(A).sum(axis=1).max() * np.abs(X).max(axis=0)))
        assert bwd <= BWD and rep.bwd_err <= BWD
        reps[refine] = rep
    if alpha == 1.0:
        assert reps[0].inner == 0, reps[0].as_dict()
    p.close()


@pytest.mark.parametrize("pinned", [False, True])
def test_streamed_host_input_equals_resident_input(ctx, pinned):
    """A mixed plan's host input streams in while the factorisation runs (the
    graph's input tasks wait for each tile column); the solution has the
    bits of the same solve on the resident input, pinned or pageable."""
    import torch
    p = t.CholPlan(ctx, 128, 8, matrix=1, alpha=1e-4, seed=5, precision=t.PREC_MIXED, mixed_kind=2)
    q = t.CholPlan(ctx, 128, 8, matrix=1, alpha=1e-2, seed=9, precision=t.PREC_MIXED, mixed_kind=2)
    host = torch.empty(q.tile_elems(), dtype=torch.float64, pin_memory=pinned)
    q.copy_tiles(1, host.data_ptr())
    B = rhs(p.N, 4, seed=13)
    for _ in range(2):  # twice: the second run's gate generation differs
        st, rep, X1 = p.solve_host(B, tiles=host.numpy())
        assert st == t.TTG_OK, rep.as_dict()
        assert rep.h2d_ms > 0 and rep.total_ms >= rep.compute_ms
        st, rep2, X2 = p.solve_host(B)  # the same input, now resident
        assert st == t.TTG_OK
        assert np.array_equal(X1, X2)
        assert rep.bwd_err == rep2.bwd_err and rep.bwd_err <= BWD
    p.close()
    q.close()
