"""bench.py's reference arm (the oracle port of the reference's CPU path on
the host cores) prints one JSON line with the keys the measurement contract
asks for.  CPU only, on a small sample."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                          "3", "--n", "1024", "--block", "128"], capture_output=True, text=True, timeout=300, cwd=ROOT,
                         check=True).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"] and d["config"]["matrix_size"] == 1024 and d["config"]["block_size"] == 128


def test_packed_host_input_matches_the_oracle():
    """The reference arm's host input equals the oracle's generated matrix."""
    import argparse
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle as orc
    a = argparse.Namespace(n=256, block=64, alpha=1e-4, seed=2)
    tiles = bench.gram_tiles_host(a)
    A = orc.gram(256, 1e-4, 2)
    ref = np.concatenate([A[i * 64:(i + 1) * 64, j * 64:(j + 1) * 64].reshape(-1, order="F") for j in range(4) for i in range(j, 4)])
    assert np.array_equal(tiles, ref)


def test_warmup_below_three_is_refused():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                        "1"], capture_output=True, text=True, timeout=60, cwd=ROOT)
    assert r.returncode != 0 and "warmup" in r.stderr
