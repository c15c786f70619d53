"""The device generator gives the oracle's bits."""
import ctypes

import numpy as np
import pytest

import tasktorrent_gb300 as t
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,stream", [(0, 0), (2, 1), (123456, 3)])
def test_normals_and_uniforms_bit_identical(ctx, seed, stream):
    import torch
    n = 100003
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    t.check(t.lib().ttg_gen_normal(ctx.h, n, seed, stream, ctypes.c_void_p(d.data_ptr()), None), "gen_normal")
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), orc.normals(0, n, seed, stream))
    t.check(t.lib().ttg_gen_uniform(ctx.h, n, seed, stream, ctypes.c_void_p(d.data_ptr()), None), "gen_uniform")
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), orc.uniforms(0, n, seed, stream))


@pytest.mark.parametrize("N,b,alpha", [(200, 40, 1e-8), (333, 64, 1.0)])
def test_gram_bit_identical(ctx, N, b, alpha):
    # Through a plan with uniform block sizes = N/b rounded; compare dense.
    nb = (N + b - 1) // b
    p = t.CholPlan(ctx, b, nb, matrix=1, alpha=alpha, seed=5)
    A = p.input_A()
    assert np.array_equal(A, orc.gram(p.N, alpha, 5))
    p.close()
