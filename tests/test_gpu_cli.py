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
