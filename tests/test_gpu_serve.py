"""The serving loop (include/ttg_serve.h): a Poisson stream of factor-and-solve
requests and follow-up right-hand sides over two executors sharing the GPU.
Every request reaches the backward-error target, and its result is the same,
bit for bit, as the same system solved alone (one-system batch, same tile
and precision): the mix does not change the answer."""
import os
import subprocess
import sys
import textwrap

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


@pytest.mark.parametrize("lanes", [1, 2])
def test_open_lanes_results_same_alone_and_in_the_mix(ctx, lanes):
    """Open lanes (admission 1): each lane's executor keeps running and takes
    a request's tasks as soon as they are published.  Every request reaches
    the target and its result is bit for bit the one-system batch's."""
    alpha, nrhs = 1e-4, 2
    s = t.Serve(36, rate=3000.0, n_min=40, n_max=700, alpha=alpha, seed=7, followup_frac=0.3, precision=t.PREC_MIXED,
                ir_steps=4, nrhs=nrhs, lanes=lanes, max_batch=6, hbm_budget_gb=2.0, keep_results=True, admission=1)
    st, rep, lat = s.run()
    assert st == t.TTG_OK, why(st)
    assert rep.completed == 36 and rep.unconverged == 0, rep.as_dict()
    assert rep.worst_bwd_err <= 1e-14 and rep.followups > 0
    assert rep.launches >= lanes  # one executor launch per epoch
    assert (lat > 0).all() and rep.p50_ms <= rep.p99_ms <= rep.max_ms
    for i in range(36):
        info = s.request(i)
        A, B, X = alone(ctx, info, alpha, t.PREC_MIXED, nrhs)
        assert np.array_equal(s.x(i), X), i
    s.close()


def test_open_lanes_tensor_core_requests_and_eviction(ctx):
    """Open lanes with tensor-core factorisations (tiles 128 and 256, team
    POTRFs) under a budget that forces evictions of resident factors."""
    s = t.Serve(24, rate=400.0, n_min=600, n_max=3000, alpha=1e-4, seed=5, followup_frac=0.4, precision=t.PREC_MIXED,
                ir_steps=3, lanes=2, max_batch=8, hbm_budget_gb=0.6, admission=1)
    st, rep, _ = s.run()
    assert st == t.TTG_OK, why(st)
    assert rep.completed == 24 and rep.unconverged == 0 and rep.worst_bwd_err <= 1e-14, rep.as_dict()
    assert rep.peak_gb <= 0.6 + 1e-9
    s.close()


def test_open_admission_rejects_bad_mode(ctx):
    with pytest.raises(t.TTGError):
        t.Serve(4, rate=100.0, precision=t.PREC_MIXED, admission=2)


def test_open_lanes_roll_over_to_new_epochs(ctx, monkeypatch):
    """An epoch whose task arena is full closes; its launch ends once its
    requests are through and the lane starts a new launch on an empty arena.
    A small arena (2048 task slots, a few requests) makes that happen often."""
    monkeypatch.setenv("TTG_SERVE_EPOCH_TASKS", "2048")
    alpha, nrhs = 1e-4, 1
    s = t.Serve(40, rate=2000.0, n_min=200, n_max=900, alpha=alpha, seed=11, followup_frac=0.3, precision=t.PREC_MIXED,
                ir_steps=3, nrhs=nrhs, lanes=2, max_batch=8, hbm_budget_gb=2.0, keep_results=True, admission=1)
    st, rep, _ = s.run()
    assert st == t.TTG_OK, why(st)
    assert rep.completed == 40 and rep.unconverged == 0 and rep.worst_bwd_err <= 1e-14, rep.as_dict()
    assert rep.launches > 4, rep.as_dict()  # more than one epoch per lane
    for i in range(0, 40, 5):
        info = s.request(i)
        A, B, X = alone(ctx, info, alpha, t.PREC_MIXED, nrhs)
        assert np.array_equal(s.x(i), X), i
    s.close()


def test_open_lanes_first_in_a_fresh_process():
    """Open lanes as the first GPU work of a process, with lazy module
    loading: the side stream's kernels (input generators, block-row scales,
    backward errors) are loaded before a lane's executor starts — a first
    launch after it would wait for an idle device that never comes."""
    code = textwrap.dedent("""
        import tasktorrent_gb300 as t
        s = t.Serve(60, rate=500.0, n_min=64, n_max=2048, alpha=1e-4, seed=2, followup_frac=0.3,
                    precision=t.PREC_MIXED, ir_steps=3, lanes=2, max_batch=16, hbm_budget_gb=8.0, admission=1)
        st, rep, _ = s.run()
        assert st == t.TTG_OK, t.strerror(st)
        assert rep.completed == 60 and rep.unconverged == 0 and rep.worst_bwd_err <= 1e-14
        s.close()
        print("ok")
    """)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, timeout=240, capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-2000:] + r.stderr[-2000:]
