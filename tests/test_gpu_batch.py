"""Batched factor-and-solve: many independent SPD systems of uneven sizes in
one executor launch (include/ttg_batch.h).  Checks each system against the
FP64 oracle (its generated matrix and numpy's solve), the backward errors,
that a system's result does not depend on what else shares the launch, and
the autotuner."""
import numpy as np
import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def why(st):
    return "%s: %s" % (t.strerror(st), t.lib().ttg_last_cuda_error().decode())


def rhs(N, nrhs, seed):
    return orc.normals(0, N * nrhs, seed, 1).reshape(N, nrhs, order="F")


def bwd(A, X, B):
    R = B - A @ X
    return np.max(np.abs(R).max(axis=0) / (np.abs(A).sum(axis=1).max() * np.abs(X).max(axis=0)))


SIZES = [1, 5, 33, 64, 100, 129, 257, 300]


@pytest.mark.parametrize("tile", [32, 64, 128])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_fp64_batch_matches_oracle(ctx, tile, nrhs):
    b = t.Batch(ctx, SIZES, tile, precision=t.PREC_F64, nrhs=nrhs, seed=3, alpha=1.0)
    st, rep = b.run()
    assert st == t.TTG_OK, why(st)
    assert rep.run.bad_runs == 0 and rep.run.tasks_pending == 0
    errs = b.backward_errors()
    for i, N in enumerate(SIZES):
        A = orc.gram(N, 1.0, 3 + i)
        B = rhs(N, nrhs, 3 + i)
        X = b.x(i)
        Xref = np.linalg.solve(A, B)
        assert np.abs(X - Xref).max() <= 1e-12 * np.abs(Xref).max(), (i, N)
        assert bwd(A, X, B) <= 1e-14
        assert errs[i] <= 1e-14
    b.close()


@pytest.mark.parametrize("ir_steps", [2, 3])
def test_mixed_batch_refines_to_fp64_backward_error(ctx, ir_steps):
    b = t.Batch(ctx, SIZES, 64, precision=t.PREC_MIXED, nrhs=2, ir_steps=ir_steps, seed=3, alpha=1.0)
    st, rep = b.run()
    assert st == t.TTG_OK, why(st)
    errs = b.backward_errors()
    assert errs.max() <= 1e-14, errs
    for i, N in enumerate(SIZES):
        A = orc.gram(N, 1.0, 3 + i)
        B = rhs(N, 2, 3 + i)
        X = b.x(i)
        assert bwd(A, X, B) <= 1e-14
        assert np.abs(X - np.linalg.solve(A, B)).max() <= 1e-12 * np.abs(X).max()
    b.close()


def test_mixed_without_refinement_is_fp32_accurate(ctx):
    b = t.Batch(ctx, [200, 333], 64, precision=t.PREC_MIXED, ir_steps=0, seed=3, alpha=1.0)
    st, _ = b.run()
    assert st == t.TTG_OK, why(st)
    e = b.backward_errors()
    assert (e > 1e-12).all() and (e < 1e-5).all()  # FP32 factor and solve, no refinement
    b.close()


@pytest.mark.parametrize("prec", [t.PREC_F64, t.PREC_MIXED])
def test_same_alone_and_in_the_mix(ctx, prec):
    """A system's solution is bit-identical whether it runs alone or with others."""
    sizes = [77, 300, 12, 256, 1, 190]
    mix = t.Batch(ctx, sizes, 64, precision=prec, nrhs=2, seed=11)
    st, _ = mix.run()
    assert st == t.TTG_OK, why(st)
    X_mix = [mix.x(i) for i in range(len(sizes))]
    mix.close()
    for i in (1, 3, 5):
        alone = t.Batch(ctx, [sizes[i]], 64, precision=prec, nrhs=2, seed=11 + i)
        st, _ = alone.run()
        assert st == t.TTG_OK, why(st)
        assert np.array_equal(alone.x(0), X_mix[i])
        alone.close()


def test_host_systems_and_repeated_runs(ctx):
    rng = np.random.default_rng(5)
    sizes = [40, 130]
    b = t.Batch(ctx, sizes, 64, precision=t.PREC_F64, nrhs=2, generate=False)
    As, Bs = [], []
    for i, N in enumerate(sizes):
        G = rng.standard_normal((N, N))
        A = G @ G.T / N + np.eye(N)
        B = rng.standard_normal((N, 2))
        b.set_system(i, A, B)
        As.append(A)
        Bs.append(B)
    outs = []
    for _ in range(3):
        st, _ = b.run()
        assert st == t.TTG_OK, why(st)
        outs.append([b.x(i) for i in range(2)])
    for i in range(2):
        assert np.array_equal(outs[0][i], outs[2][i])  # each run starts from the inputs
        assert np.abs(outs[0][i] - np.linalg.solve(As[i], Bs[i])).max() <= 1e-12 * np.abs(outs[0][i]).max()
    b.close()


def test_autotune_picks_a_measured_configuration(ctx):
    rng = np.random.default_rng(1)
    sizes = np.exp(rng.uniform(np.log(32), np.log(512), 60)).astype(np.int32)
    full = t.lib().ttg_workers(ctx.h)
    tile, workers, ms = t.batch_autotune(ctx, sizes, [64, 128], [0, max(1, full // 2)], max_sample=30)
    assert tile in (64, 128) and 1 <= workers <= full and ms > 0
    t.check(t.lib().ttg_set_workers(ctx.h, 0), "reset workers")
