"""The FP64-accurate tensor-core product (ttg_sliced_matmul) against an
extended-precision reference, and the refinement with sliced residuals
against the FP64 ones.

Bound: every entry of Y = T·X is within 2^-50 · (|T|·|X|) of the exact value
(computed in numpy's long double); the FP64 FMA product of the same size is
typically off by ~sqrt(N)·2^-53 · (|T|·|X|)."""
import ctypes

import numpy as np
import pytest

import tasktorrent_gb300 as t

pytestmark = pytest.mark.gpu
REL = 2.0 ** -50


def sliced(ctx, T, X, B=None):
    """Y = T @ X (or B - T @ X) on the device: T row-major N×N is the
    column-major Tᵀ, so the product Aᵀ·X of the entry point is T·X."""
    import torch
    N, nrhs = X.shape
    dT = torch.from_numpy(np.ascontiguousarray(T)).cuda()
    dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()  # (nrhs, N) row-major = N×nrhs column-major
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda() if B is not None else None
    dY = torch.empty_like(dX)
    st = t.lib().ttg_sliced_matmul(ctx.h, N, ctypes.c_void_p(dT.data_ptr()), nrhs, ctypes.c_void_p(dX.data_ptr()),
                                   ctypes.c_void_p(dB.data_ptr()) if dB is not None else None,
                                   ctypes.c_void_p(dY.data_ptr()), 2 if B is not None else 0, None)
    assert st == t.TTG_OK, t.strerror(st)
    torch.cuda.synchronize()
    return dY.cpu().numpy().T


def exact(T, X, B=None):
    ld = np.longdouble
    Y = T.astype(ld) @ X.astype(ld)
    if B is not None:
        Y = B.astype(ld) - Y
    return Y


def check(Y, T, X, B=None, rel=REL):
    ref = exact(T, X, B)
    bound = np.abs(T).astype(np.longdouble) @ np.abs(X).astype(np.longdouble)
    err = np.abs(Y.astype(np.longdouble) - ref)
    # The subtraction B − T·X rounds once more (half an ulp of the result).
    slack = np.abs(ref) * 2.0 ** -53 if B is not None else 0
    assert np.all(err <= rel * bound + slack), float(np.max(err / np.maximum(bound, 1e-300)))


@pytest.mark.parametrize("N,nrhs", [(512, 16), (1000, 5), (333, 1), (1280, 16)])
def test_sliced_product_is_fp64_accurate(ctx, N, nrhs):
    rng = np.random.default_rng(N + nrhs)
    T = rng.standard_normal((N, N))
    X = rng.standard_normal((N, nrhs))
    check(sliced(ctx, T, X), T, X)


def test_sliced_residual_mode(ctx):
    rng = np.random.default_rng(5)
    N, nrhs = 768, 16
    G = rng.standard_normal((N, N))
    A = G @ G.T / N + 1e-4 * np.eye(N)
    X = rng.standard_normal((N, nrhs))
    B = A @ X + 1e-12 * rng.standard_normal((N, nrhs))  # a residual far below ‖B‖
    check(sliced(ctx, A, X, B), A, X, B)


def test_sliced_product_scales_zeros_and_signs(ctx):
    """Rows and columns spanning 2^±300, a zero row, a zero column, and
    equal entries (the largest digit in every position)."""
    rng = np.random.default_rng(9)
    N, nrhs = 640, 7
    T = rng.standard_normal((N, N)) * np.exp2(rng.integers(-300, 300, N))[:, None]
    T[17, :] = 0.0
    T[40:60, :] = 0.49999999999999994  # just below 1/2: first digit 128
    X = rng.standard_normal((N, nrhs)) * np.exp2(rng.integers(-200, 200, nrhs))[None, :]
    X[:, 3] = 0.0
    X[:, 5] = -0.49999999999999994
    Y = sliced(ctx, T, X)
    assert np.all(Y[17] == 0.0) and np.all(Y[:, 3] == 0.0)
    check(Y, T, X)


def test_sliced_product_is_deterministic(ctx):
    rng = np.random.default_rng(3)
    T = rng.standard_normal((1024, 1024))
    X = rng.standard_normal((1024, 16))
    assert np.array_equal(sliced(ctx, T, X), sliced(ctx, T, X))


@pytest.mark.parametrize("alpha", [1.0, 1e-4, 1e-8])
def test_refinement_with_sliced_residuals(ctx, alpha):
    """GMRES-IR with the sliced residuals reaches the same backward error as
    with FP64 FMA residuals, and the solution agrees with numpy's."""
    b, nb, nrhs = 128, 6, 8
    rng = np.random.default_rng(7)
    outs = {}
    for res in (1, 2):
        p = t.CholPlan(ctx, b, nb, matrix=1, alpha=alpha, seed=2, precision=t.PREC_MIXED, mixed_kind=2)
        A = p.input_A()
        B = rng.standard_normal((p.N, nrhs)) if res == 1 else outs[1][2]
        st, rep, X = p.solve_host(B, tol=1e-14, max_outer=12, restart=30, residual=res)
        p.close()
        assert st == t.TTG_OK, (res, rep.as_dict())
        R = B - A @ X
        bwd = np.max(np.abs(R).max(axis=0) / (np.abs(A).sum(axis=1).max() * np.abs(X).max(axis=0)))
        assert bwd <= 1e-14 and rep.bwd_err <= 1e-14
        outs[res] = (X, rep, B, A)
    X1, X2, A = outs[1][0], outs[2][0], outs[1][3]
    Xr = np.linalg.solve(A, outs[1][2])
    cond = np.linalg.cond(A)
    assert np.linalg.norm(X2 - Xr) / np.linalg.norm(Xr) <= 1e-15 * cond * 50
