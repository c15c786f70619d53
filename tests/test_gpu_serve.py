"""The serving loop (include/ttg_serve.h): a Poisson stream of factor-and-solve
requests and follow-up right-hand sides over two executors sharing the GPU.
Every request reaches the backward-error target, and its result is the same,
bit for bit, as the same system solved alone (one-system batch, same tile
and precision): the mix does not change the answer."""
import numpy as np
import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def why(st):
    return "%s: %s" % (t.strerror(st), t.lib().ttg_last_cuda_error().decode())


def alone(ctx, info, alpha, precision, nrhs):
    N = info["n"]
    A = orc.gram(N, alpha, info["seed_a"])
    B = orc.normals(0, N * nrhs, info["seed_b"], 1).reshape(N, nrhs, order="F")
    b = t.Batch(ctx, [N], info["tile"], precision=precision, nrhs=nrhs, ir_steps=info["ir_steps"], generate=False)
    b.set_system(0, A, B)
    st, _ = b.run()
    assert st == t.TTG_OK, why(st)
    X = b.x(0)
    b.close()
    return A, B, X


@pytest.mark.parametrize("precision", [t.PREC_F64, t.PREC_MIXED])
def test_stream_results_same_alone_and_in_the_mix(ctx, precision):
    alpha, nrhs = 1e-4, 2
    s = t.Serve(36, rate=3000.0, n_min=40, n_max=700, alpha=alpha, seed=7, followup_frac=0.3, precision=precision,
                ir_steps=4, nrhs=nrhs, lanes=2, max_batch=6, hbm_budget_gb=2.0, keep_results=True)
    st, rep, lat = s.run()
    assert st == t.TTG_OK, why(st)
    assert rep.completed == 36 and rep.unconverged == 0, rep.as_dict()
    assert rep.worst_bwd_err <= 1e-14 and rep.followups > 0 and rep.launches > 1
    assert (lat > 0).all() and rep.p50_ms <= rep.p99_ms <= rep.max_ms
    for i in range(36):
        info = s.request(i)
        A, B, X = alone(ctx, info, alpha, precision, nrhs)
        Xs = s.x(i)
        assert np.array_equal(Xs, X), i
        R = B - A @ Xs
        be = np.max(np.abs(R).max(axis=0) / (np.abs(A).sum(axis=1).max() * np.abs(Xs).max(axis=0)))
        assert be <= 1e-14 and info["bwd_err"] <= 1e-14
    s.close()


def test_small_budget_evicts_and_refactors(ctx):
    s = t.Serve(40, rate=5000.0, n_min=200, n_max=400, alpha=1e-4, seed=3, followup_frac=0.5, precision=t.PREC_MIXED,
                ir_steps=4, lanes=2, max_batch=4, hbm_budget_gb=0.012)
    st, rep, _ = s.run()
    assert st == t.TTG_OK, why(st)
    assert rep.completed == 40 and rep.unconverged == 0
    assert rep.evictions > 0 and rep.peak_gb <= 0.012 + 1e-9
    s.close()


def test_budget_below_one_request_is_reported(ctx):
    s = t.Serve(3, rate=1000.0, n_min=2000, n_max=2000, precision=t.PREC_F64, hbm_budget_gb=0.001)
    st, _, _ = s.run()
    assert st == t.TTG_ENOMEM
    s.close()
