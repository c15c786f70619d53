"""Row-vector tile operations (m <= 16 right-hand-side rows) used by the block
triangular solves of the batched path: GEMM_NT / GEMM_NN / TRSM_RLTN /
TRSM_RLNN with few rows, and the precision-converting CONVERT, in FP64 and in
FP32 (TTG_PREC_MIXED), against numpy."""
import numpy as np
import pytest

import tasktorrent_gb300 as t

pytestmark = pytest.mark.gpu


def _dev(a, dtype=np.float64):
    """Device copy of `a`, column-major; returns (tensor, ptr)."""
    import torch
    tt = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dtype).T)).cuda()
    return tt, tt.data_ptr()


def _back(tt, shape):
    return tt.cpu().numpy().T.reshape(shape).astype(np.float64)


def _run(ctx, op):
    t.check(ctx.upload([op], np.zeros(1, np.int32), np.zeros(2, np.int64), np.zeros(0, np.int32)), "upload")
    return ctx.run()


def _lower(n, rng):
    G = rng.standard_normal((n, n))
    return np.linalg.cholesky(G @ G.T / n + np.eye(n))


@pytest.mark.parametrize("prec", [t.PREC_F64, t.PREC_MIXED])
@pytest.mark.parametrize("parts", [0, 1, 3])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (1, 512, 512), (3, 100, 77), (16, 300, 40), (5, 1000, 17)])
def test_gemm_small_m(ctx, prec, parts, m, n, k):
    import torch
    dt = np.float64 if prec == t.PREC_F64 else np.float32
    tol = 1e-13 if prec == t.PREC_F64 else 2e-5
    rng = np.random.default_rng(m * 7 + n + k)
    A = rng.standard_normal((m, k))
    C0 = rng.standard_normal((m, n))
    for kind, B in ((t.OP_GEMM_NT, rng.standard_normal((n, k))), (t.OP_GEMM_NN, rng.standard_normal((k, n)))):
        ref = C0 - A @ (B.T if kind == t.OP_GEMM_NT else B)
        dA, pA = _dev(A, dt)
        dB, pB = _dev(B, dt)
        dC, pC = _dev(C0, dt)
        torch.cuda.synchronize()
        op = t.Op(kind=kind, prec=prec, m=m, n=n, k=k, lda=m, ldb=B.shape[0], ldc=m, parts=parts, alpha=-1.0, beta=1.0,
                  a=pA, b=pB, c=pC)
        st, _ = _run(ctx, op)
        assert st == t.TTG_OK
        got = _back(dC, (m, n))
        assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max()) * np.sqrt(k)


@pytest.mark.parametrize("prec", [t.PREC_F64, t.PREC_MIXED])
@pytest.mark.parametrize("kind", [t.OP_TRSM_RLTN, t.OP_TRSM_RLNN])
@pytest.mark.parametrize("m,n,alpha,parts", [(1, 1, 1.0, 0), (1, 512, 1.0, 0), (5, 33, -0.5, 0), (16, 300, 1.0, 0),
                                             (40, 70, 2.0, 3)])
def test_trsm_small_m(ctx, prec, kind, m, n, alpha, parts):
    import torch
    dt = np.float64 if prec == t.PREC_F64 else np.float32
    tol = 1e-12 if prec == t.PREC_F64 else 1e-4
    rng = np.random.default_rng(m + 11 * n)
    L = _lower(n, rng)
    B = rng.standard_normal((m, n))
    ref = alpha * (B @ np.linalg.inv(L).T if kind == t.OP_TRSM_RLTN else B @ np.linalg.inv(L))
    dL, pL = _dev(L, dt)
    dB, pB = _dev(B, dt)
    torch.cuda.synchronize()
    op = t.Op(kind=kind, prec=prec, m=m, n=n, lda=n, ldc=m, parts=parts, alpha=alpha, a=pL, c=pB)
    st, _ = _run(ctx, op)
    assert st == t.TTG_OK
    got = _back(dB, (m, n))
    assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
@pytest.mark.parametrize("beta", [0.0, 1.0])
def test_convert(ctx, flags, beta):
    import torch
    rng = np.random.default_rng(flags + 10)
    m, n = 37, 21
    A = rng.standard_normal((m, n))
    C0 = rng.standard_normal((m, n))
    adt = np.float32 if flags & 1 else np.float64
    cdt = np.float32 if flags & 2 else np.float64
    dA, pA = _dev(A, adt)
    dC, pC = _dev(C0, cdt)
    torch.cuda.synchronize()
    op = t.Op(kind=t.OP_CONVERT, m=m, n=n, lda=m, ldc=m, flags=flags, alpha=-2.0, beta=beta, a=pA, c=pC)
    st, _ = _run(ctx, op)
    assert st == t.TTG_OK
    ref = -2.0 * A.astype(adt).astype(np.float64) + beta * C0.astype(cdt).astype(np.float64)
    got = _back(dC, (m, n))
    tol = 1e-6 if cdt == np.float32 else 1e-15
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
