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
