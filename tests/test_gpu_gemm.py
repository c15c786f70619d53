"""2D block GEMM task graph on the GPU against the oracle: exact on the
reference's integer inputs (val_global), ≤ 1e-12 relative Frobenius on
U[-1,1] inputs, and the same DAG as the reference runtime."""
import os

import numpy as np
import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("N,b", [(64, 4), (512, 64), (1024, 256)])
def test_val_global_exact(ctx, N, b):
    p = t.GemmPlan(ctx, N, b, inputs=0)
    st, rep = p.run()
    assert st == t.TTG_OK and rep.tasks_run == 2 * (N // b) ** 2 + (N // b) ** 3
    A, _ = orc.gemm_inputs(N, 0, 0)
    Ai = A.astype(np.int64)
    assert np.array_equal(p.C(), (Ai @ Ai).astype(np.float64))
    p.close()


@pytest.mark.parametrize("N,b", [(256, 32), (1024, 512)])
def test_uniform_matches_oracle(ctx, N, b):
    p = t.GemmPlan(ctx, N, b, inputs=1, seed=1)
    st, rep = p.run()
    assert st == t.TTG_OK
    r = orc.gemm(N, b, n_threads=8, inputs=1, seed=1)
    C = p.C()
    assert np.linalg.norm(C - r["C"]) <= 1e-12 * np.linalg.norm(r["C"])
    p.close()


def test_device_dag_equals_reference_runtime(ctx, tmp_path):
    p = t.GemmPlan(ctx, 64, 4, n_threads=4, inputs=1)
    st, rep = p.run()
    assert st == t.TTG_OK
    pre = str(tmp_path / "g")
    p.dump_dag(pre)
    assert orc.read_dag(pre) == orc.read_dag(os.path.join(GOLDEN, "dag_gemm_nb16"))
    p.close()


def test_host_path(ctx):
    N, b = 256, 64
    p = t.GemmPlan(ctx, N, b, inputs=1, seed=1)
    A, B = orc.gemm_inputs(N, 1, 1)
    st, rep, C = p.host(A, B)
    assert st == t.TTG_OK
    assert np.linalg.norm(C - A @ B) <= 1e-12 * np.linalg.norm(A @ B)
    p.close()
