"""The 2d_cholesky / 2d_gemm command lines with the reference's flags."""
import os
import subprocess

import pytest

import tasktorrent_gb300 as t

pytestmark = pytest.mark.gpu


def run(prog, *args):
    r = subprocess.run([os.path.join(t.BIN_DIR, prog)] + list(args), capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout + r.stderr


def test_cholesky_defaults_self_test():
    rc, out = run("2d_cholesky")
    assert rc == 0, out
    assert "=> Error solve" in out and ">>>>" in out


@pytest.mark.parametrize("args", [["--block_size=64", "--num_blocks=8", "--kind=2"],
                                  ["--block_size=10", "--num_blocks=12", "--accumulate=true", "--upper_block_size=15"],
                                  ["--block_size=128", "--num_blocks=16", "--matrix=gram", "--test=true"]])
def test_cholesky_variants(args):
    rc, out = run("2d_cholesky", *args)
    assert rc == 0, out
    err = float(out.split("=> Error solve")[1].split()[0])
    assert err <= 1e-6


def test_gemm_defaults_exact():
    rc, out = run("2d_gemm")
    assert rc == 0, out
    err = float(out.split("==> GEMM error")[1].split()[0])
    assert err == 0.0


def field_line(out, tag):
    lines = [l for l in out.splitlines() if l.startswith(tag)]
    assert lines, out
    return lines[-1].split()


@pytest.mark.parametrize("args", [["4", "2000", "1e-5", "1", "2"], ["4", "500", "0", "0", "1"]])
def test_ttor_wait(args):
    """The reference's wait-only micro-benchmark: every task runs, and the
    efficiency n_tasks·spin/(time·workers) is a fraction."""
    rc, out = run("ttor_wait", *args)
    assert rc == 0, out
    f = field_line(out, ">>>>")
    # >>>> exp repeat n_threads spin_time n_tasks efficiency_mean ...
    assert f[1] == "ttor_wait_time_insertion" + args[3] and int(f[2]) == int(args[4])
    assert int(f[5]) == int(args[1])
    eff = float(f[6])
    assert 0.0 <= eff <= 1.05
    if float(args[2]) > 0:
        dev = [float(l.split()[5]) for l in out.splitlines() if l.startswith("####")]
        assert dev and all(0.0 < e <= 1.05 for e in dev), out


def test_ttor_deps():
    """The reference's dependency-chain micro-benchmark: n_rows × n_cols tasks
    with n_edges promises each from inside the task bodies."""
    rc, out = run("ttor_deps", "4", "64", "8", "20", "2e-5", "2")
    assert rc == 0, out
    f = field_line(out, ">>>>")
    # >>>> ttor_deps repeat n_threads n_rows n_edges n_cols spin_time n_tasks eff_mean eff_std time_mean time_std
    assert f[1] == "ttor_deps" and int(f[4]) == 64 and int(f[5]) == 8 and int(f[6]) == 20 and int(f[8]) == 64 * 20
    assert 0.0 < float(f[9]) <= 1.05


def test_log_and_deps_files_parse_like_the_reference_tool(tmp_path):
    """2d_cholesky --log / --depslog write the reference's trace files
    (2d_cholesky.cpp:630-644); they are read here the way
    tools/ttor_logging.py:11-25 reads them: three columns what,time_start,
    time_end, rows containing '>run>', task = third '>' field, kind = the
    task name before its first '_'; and the dependency file's two columns."""
    import csv
    r = subprocess.run([os.path.join(t.BIN_DIR, "2d_cholesky"), "--block_size=32", "--num_blocks=16", "--n_threads=4",
                        "--kind=2", "--log=true", "--depslog=true"], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    log = tmp_path / "ttor_dist_32_16_1_4_2.log.0"
    deps = tmp_path / "deps_ttor_dist_32_16_1_4_2.dot.0"
    rows = [row for row in csv.reader(open(log)) if len(row) == 3 and ">run>" in row[0] and "intern" not in row[0]]
    tasks = [row[0].split(">")[2] for row in rows]
    kinds = {}
    for k in (name.split("_")[0] for name in tasks):
        kinds[k] = kinds.get(k, 0) + 1
    assert len(tasks) == 816 == len(set(tasks))  # nb = 16: 16 + 120 + 680 tasks, each once
    assert kinds == {"POTRF": 16, "TRSM": 120, "GEMM": 680}
    starts, ends = [float(row[1]) for row in rows], [float(row[2]) for row in rows]
    assert all(e >= s for s, e in zip(starts, ends))
    assert all(row[0].startswith("Wk_Chol_0_") for row in rows)
    edges = [tuple(row) for row in csv.reader(open(deps)) if row]
    names = set(tasks)
    assert all(len(e) == 2 and e[0] in names and e[1] in names for e in edges)
    preds = {}
    for a, b in edges:
        preds[b] = preds.get(b, 0) + 1
    # A task's predecessors are its indegree (2d_cholesky.cpp:346-353, 449-456,
    # 534-541); the first POTRF is seeded by the main thread.
    assert "POTRF_0" not in preds
    assert preds["TRSM_1_0"] == 1 and preds["TRSM_2_1"] == 2 and preds["GEMM_0_1_1"] == 1 and preds["GEMM_1_2_2"] == 2
    assert preds["GEMM_1_3_2"] == 3 and preds["POTRF_1"] == 1
