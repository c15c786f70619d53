"""Generate the golden fixtures of tests/golden/ from the REFERENCE's own
runtime (ttor::Taskflow + ttor::Threadpool_shared compiled from the reference
sources into oracle/_ref by oracle/Makefile).

Run in a container that has the reference tree (oracle/Makefile's REF, or --ref):

    python tests/golden/make_golden.py [--ref /path/to/reference]

Fixtures written (all small):
  dag_chol_nb16_k{0,2}_acc{0,1}.{tasks,edges}.csv.gz  Cholesky DAG, 16×16 tiles
  dag_gemm_nb16.{tasks,edges}.csv.gz                  block GEMM DAG, 16×16 tiles
  chol_gram_n256_b32.json   column sums / sums of squares of L (plain-loop BLAS)
  gemm_unif_n128_b32.json   column sums of C = A·B (plain-loop BLAS)
  ttor_cholesky_nb16.json   task count printed by the reference's ttor_cholesky
"""
import argparse
import gzip
import json
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")


def gz(src, dst):
    with open(src, "rb") as f, open(dst, "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
            g.write(f.read())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference tree (default: oracle/Makefile's REF)")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "ref"] + (["REF=" + a.ref] if a.ref else []), cwd=ORACLE, check=True)
    ref_dag = os.path.join(ORACLE, "_ref", "ref_dag")
    env = dict(os.environ)
    env.pop("TTG_ORACLE_BLAS", None)  # plain loops: bit-reproducible on any host
    tmp = tempfile.mkdtemp()
    try:
        for kind in (0, 2):
            for acc in (0, 1):
                pre = os.path.join(tmp, "c")
                subprocess.run([ref_dag, "cholesky", "4", "4", "16", str(kind), str(acc), "-1", "0", "1", "0", pre],
                               check=True, env=env, capture_output=True)
                name = "dag_chol_nb16_k%d_acc%d" % (kind, acc)
                gz(pre + ".tasks.csv", os.path.join(HERE, name + ".tasks.csv.gz"))
                gz(pre + ".edges.csv", os.path.join(HERE, name + ".edges.csv.gz"))
        pre = os.path.join(tmp, "g")
        subprocess.run([ref_dag, "gemm", "4", "64", "4", "1", "1", pre], check=True, env=env, capture_output=True)
        gz(pre + ".tasks.csv", os.path.join(HERE, "dag_gemm_nb16.tasks.csv.gz"))
        gz(pre + ".edges.csv", os.path.join(HERE, "dag_gemm_nb16.edges.csv.gz"))

        lbin = os.path.join(tmp, "L.bin")
        subprocess.run([ref_dag, "cholesky", "4", "32", "8", "2", "0", "-1", "1", "1.0", "0", os.path.join(tmp, "n"), lbin],
                       check=True, env=env, capture_output=True)
        L = np.fromfile(lbin, dtype=np.float64).reshape(256, 256, order="F")
        with open(os.path.join(HERE, "chol_gram_n256_b32.json"), "w") as f:
            json.dump({"N": 256, "block_size": 32, "matrix": "gram", "alpha": 1.0, "seed": 0,
                       "colsum": [float.hex(float(v)) for v in L.sum(axis=0)],
                       "colsq": [float.hex(float(v)) for v in (L * L).sum(axis=0)]}, f, indent=0)
        cbin = os.path.join(tmp, "C.bin")
        subprocess.run([ref_dag, "gemm", "4", "128", "32", "1", "1", os.path.join(tmp, "m"), cbin], check=True, env=env,
                       capture_output=True)
        C = np.fromfile(cbin, dtype=np.float64).reshape(128, 128, order="F")
        with open(os.path.join(HERE, "gemm_unif_n128_b32.json"), "w") as f:
            json.dump({"N": 128, "block_size": 32, "inputs": "uniform", "seed": 1,
                       "colsum": [float.hex(float(v)) for v in C.sum(axis=0)]}, f, indent=0)
        r = subprocess.run([os.path.join(ORACLE, "_ref", "ttor_cholesky"), "4", "16", "0", "0"], check=True,
                           capture_output=True, text=True)
        fields = r.stdout.strip().split(",")
        with open(os.path.join(HERE, "ttor_cholesky_nb16.json"), "w") as f:
            json.dump({"n_threads": int(fields[0]), "n_blocks": int(fields[1]), "total_tasks": int(fields[4])}, f)
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
