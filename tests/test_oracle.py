"""The oracle against the golden fixtures made from the reference's own
runtime (tests/golden/make_golden.py), and the seeded generator against
published known answers.  CPU only."""
import gzip
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_philox_known_answers():
    # Published Philox-4x32-10 known-answer vectors (Salmon et al., Random123).
    assert orc.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_box_muller_matches_libm():
    # The portable log / sincos of ttg_philox.h agree with libm to ~1e-15.
    seed, stream, n = 7, 1, 4000
    z = orc.normals(0, 2 * n, seed, stream)
    for c in range(0, n, 97):
        r = orc.philox([c, 0, 0, 0], [seed, stream])
        k1 = ((r[0] << 32) | r[1]) >> 11
        k2 = ((r[2] << 32) | r[3]) >> 11
        u1 = (k1 + 0.5) * 2.0 ** -53
        u2 = (k2 + 0.5) * 2.0 ** -53
        rad = np.sqrt(-2.0 * np.log(u1))
        assert abs(z[2 * c] - rad * np.cos(2 * np.pi * u2)) <= 1e-13 * (1 + abs(z[2 * c]))
        assert abs(z[2 * c + 1] - rad * np.sin(2 * np.pi * u2)) <= 1e-13 * (1 + abs(z[2 * c + 1]))


def test_generator_statistics():
    z = orc.normals(0, 400000, 0, 0)
    assert abs(z.mean()) < 0.01 and abs(z.var() - 1) < 0.01
    u = orc.uniforms(0, 400000, 1, 2)
    assert -1 <= u.min() and u.max() <= 1 and abs(u.mean()) < 0.01 and abs(u.var() - 1 / 3) < 0.01
    q = orc.qnormals(0, 400000, 0, 0)
    assert q.min() >= -127 and q.max() <= 127 and abs((q / 16.0).var() - 1) < 0.01


def test_gram_is_exact():
    # A = G·Gᵀ/N + αI from integer G: compare with an int64 product.
    N, alpha, seed = 96, 1e-4, 2
    A = orc.gram(N, alpha, seed)
    g = orc.qnormals(0, N * N, seed, 0).reshape(N, N, order="F").astype(np.int64)
    S = g @ g.T
    ref = S.astype(np.float64) / (256.0 * N) + alpha * np.eye(N)
    assert np.array_equal(A, ref)
    assert np.array_equal(A, A.T)


def _golden(name):
    return orc.read_dag(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("kind,acc", [(0, 0), (0, 1), (2, 0), (2, 1)])
def test_oracle_cholesky_dag_matches_reference_runtime(tmp_path, kind, acc):
    pre = str(tmp_path / "o")
    r = orc.cholesky(block_size=4, num_blocks=16, n_threads=4, kind=kind, accumulate=bool(acc), matrix=0, want_L=False,
                     dag_prefix=pre)
    assert r["errors"] == 0
    assert orc.read_dag(pre) == _golden("dag_chol_nb16_k%d_acc%d" % (kind, acc))


def test_oracle_gemm_dag_matches_reference_runtime(tmp_path):
    pre = str(tmp_path / "g")
    r = orc.gemm(64, 4, n_threads=4, dag_prefix=pre, want_C=False)
    assert r["errors"] == 0
    assert orc.read_dag(pre) == _golden("dag_gemm_nb16")


def test_task_counts():
    # potrf nb + trsm nb(nb-1)/2 + gemm (nb-1)nb(nb+1)/6; 816 at nb = 16, as
    # the reference's ttor_cholesky prints.
    tasks, _ = _golden("dag_chol_nb16_k0_acc0")
    with open(os.path.join(GOLDEN, "ttor_cholesky_nb16.json")) as f:
        assert len(tasks) == json.load(f)["total_tasks"] == 16 + 120 + 680
    tasks, edges = _golden("dag_gemm_nb16")
    assert len(tasks) == 2 * 256 + 4096
    assert all(v[1] == v[0] and v[2] == 1 for v in tasks.values())


def test_oracle_cholesky_factor_matches_reference_runtime():
    with open(os.path.join(GOLDEN, "chol_gram_n256_b32.json")) as f:
        g = json.load(f)
    r = orc.cholesky(block_size=32, num_blocks=8, n_threads=4, kind=2, matrix=1, alpha=1.0, seed=0, want_A=True)
    assert r["blas"] == "loops"
    L = r["L"]
    assert [float.hex(float(v)) for v in L.sum(axis=0)] == g["colsum"]
    assert [float.hex(float(v)) for v in (L * L).sum(axis=0)] == g["colsq"]
    A = r["A"]
    assert np.linalg.norm(L @ L.T - A) / np.linalg.norm(A) < 1e-15


def test_oracle_gemm_matches_reference_runtime():
    with open(os.path.join(GOLDEN, "gemm_unif_n128_b32.json")) as f:
        g = json.load(f)
    r = orc.gemm(128, 32, n_threads=3, inputs=1, seed=1)
    assert [float.hex(float(v)) for v in r["C"].sum(axis=0)] == g["colsum"]
    A, B = orc.gemm_inputs(128, 1, 1)
    assert np.allclose(r["C"], A @ B, rtol=0, atol=1e-12)


def test_oracle_gemm_val_global_exact():
    # Integer inputs: any summation order gives the exact product.
    r = orc.gemm(96, 16, n_threads=4, inputs=0)
    A, _ = orc.gemm_inputs(96, 0, 0)
    Ai = A.astype(np.int64)
    assert np.array_equal(r["C"], (Ai @ Ai).astype(np.float64))


@pytest.mark.parametrize("upper", [-1, 7])
@pytest.mark.parametrize("acc", [False, True])
def test_oracle_cholesky_uneven_and_accumulate(upper, acc):
    r = orc.cholesky(block_size=5, num_blocks=10, n_threads=3, kind=3, accumulate=acc, upper_block_size=upper, matrix=0,
                     want_A=True)
    L, A = r["L"], r["A"]
    assert r["errors"] == 0 and r["info"] == 0
    assert np.linalg.norm(L @ L.T - A) / np.linalg.norm(A) < 1e-13


def test_oracle_reports_non_spd():
    # alpha = -1 makes the gram matrix indefinite: dpotrf's info is reported.
    r = orc.cholesky(block_size=8, num_blocks=4, n_threads=2, matrix=1, alpha=-1.0, seed=0)
    assert r["info"] > 0


@pytest.mark.skipif(not os.path.exists(orc.REF_DAG), reason="oracle/_ref is only built where the reference tree is present")
@pytest.mark.parametrize("args", [("3", "5", "10", "1", "0", "7"), ("2", "6", "9", "3", "1", "9"), ("5", "4", "7", "2", "0", "-1")])
def test_restated_runtime_equals_reference_runtime(tmp_path, args):
    """The oracle's restated runtime and the reference's own runtime give the
    same DAG and the same factor (plain-loop BLAS) on more configurations."""
    import subprocess
    nt, b, nb, kind, acc, upper = args
    pre_ref = str(tmp_path / "r")
    lbin = str(tmp_path / "L.bin")
    env = dict(os.environ)
    env.pop("TTG_ORACLE_BLAS", None)
    subprocess.run([orc.REF_DAG, "cholesky", nt, b, nb, kind, acc, upper, "1", "0.5", "3", pre_ref, lbin], check=True, env=env,
                   capture_output=True)
    pre = str(tmp_path / "o")
    r = orc.cholesky(block_size=int(b), num_blocks=int(nb), n_threads=int(nt), kind=int(kind), accumulate=bool(int(acc)),
                     upper_block_size=int(upper), matrix=1, alpha=0.5, seed=3, dag_prefix=pre)
    assert orc.read_dag(pre) == orc.read_dag(pre_ref)
    Lref = np.fromfile(lbin).reshape(r["N"], r["N"], order="F")
    if acc == "0":
        # Each tile's updates run in the fixed k order of the chain: bit-exact.
        assert np.array_equal(r["L"], Lref)
    else:
        # The accumulate flow adds partial products in arrival order.
        assert np.linalg.norm(r["L"] - Lref) <= 1e-14 * np.linalg.norm(Lref)


def _pack_lower_tiles(A, sizes):
    """Packed lower tiles of A in the device layout: tile (i,j), i >= j, column
    of tiles after column of tiles, each column-major."""
    displ = np.concatenate([[0], np.cumsum(sizes)])
    parts = []
    for j in range(len(sizes)):
        for i in range(j, len(sizes)):
            parts.append(A[displ[i]:displ[i + 1], displ[j]:displ[j + 1]].reshape(-1, order="F"))
    return np.concatenate(parts)


def test_packed_tile_input_equals_generated_input():
    """matrix 2 (packed tiles given) factors the same input to the same bits."""
    b, nb = 32, 6
    r1 = orc.cholesky(block_size=b, num_blocks=nb, n_threads=4, kind=2, matrix=1, alpha=1e-4, seed=2, want_A=True)
    tiles = _pack_lower_tiles(r1["A"], orc.block_sizes(b, nb))
    r2 = orc.cholesky(block_size=b, num_blocks=nb, n_threads=4, kind=2, tiles=tiles, want_A=True)
    assert np.array_equal(r1["A"], r2["A"])
    assert np.array_equal(r1["L"], r2["L"])
    N = b * nb
    assert r1["flops"] == pytest.approx(N ** 3 / 3.0, rel=1e-12)


@pytest.mark.parametrize("limit", [1, 2, 3])
def test_panel_limited_sample(limit):
    """panel_limit P runs the tasks of the first P panel steps: their count and
    flops follow the task formulas, and the first P tile columns are final."""
    b, nb = 16, 6
    full = orc.cholesky(block_size=b, num_blocks=nb, n_threads=4, kind=2, matrix=1, alpha=1.0, seed=0)
    part = orc.cholesky(block_size=b, num_blocks=nb, n_threads=4, kind=2, matrix=1, alpha=1.0, seed=0, panel_limit=limit)
    tasks = sum(1 + (nb - 1 - j) for j in range(limit)) + sum((nb - k - 1) * (nb - k) // 2 for k in range(limit))
    assert part["tasks"] == tasks and part["errors"] == 0 and part["info"] == 0
    flops = sum(b ** 3 / 3 + (nb - 1 - j) * b ** 3 for j in range(limit))
    for k in range(limit):
        m = nb - k - 1  # trailing tile rows
        flops += m * b ** 3 + m * (m - 1) // 2 * 2 * b ** 3  # SYRKs + GEMMs of panel step k
    assert part["flops"] == pytest.approx(flops, rel=1e-12)
    c = limit * b
    assert np.array_equal(part["L"][:, :c], full["L"][:, :c])


def test_gram_entry_equals_whole_matrix():
    """One entry computed alone (the bench's spot check of a large input)
    equals the same entry of the whole generated matrix."""
    A = orc.gram(96, 1e-4, 2)
    for i, j in [(0, 0), (95, 0), (50, 17), (95, 95), (33, 32)]:
        assert orc.gram_entry(96, i, j, 1e-4, 2) == A[i, j]
