/*
 * ref_driver.cpp — TEST INFRASTRUCTURE ONLY.  Runs the oracle's task graphs
 * (dag.hpp) on the REFERENCE's own runtime, ttor::Taskflow<K> and
 * ttor::Threadpool_shared compiled from the reference's sources
 * (tasktorrent/src/{tasks,threadpool_shared,util}.cpp with -DTTOR_SHARED) by
 * oracle/Makefile into oracle/_ref/.  It writes the DAG record and the factor
 * that the golden fixtures under tests/golden/ are made from.
 *
 *   ref_dag cholesky <n_threads> <block> <num_blocks> <kind> <accumulate> <upper> <matrix> <alpha> <seed> <prefix> [L.bin]
 *   ref_dag gemm <n_threads> <N> <block> <inputs> <seed> <prefix> [C.bin]
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tasktorrent/tasktorrent.hpp"
#include "dag.hpp"

template <class K>
using RefFlow = ttor::Taskflow<K>;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string what = argv[1];
    if (what == "cholesky" && argc >= 12) {
        orc_chol_args a{};
        a.n_threads = atoi(argv[2]);
        a.block_size = atoi(argv[3]);
        a.num_blocks = atoi(argv[4]);
        a.prio_kind = atoi(argv[5]);
        a.accumulate = atoi(argv[6]);
        a.upper_block_size = atoi(argv[7]);
        a.matrix = atoi(argv[8]);
        a.alpha = atof(argv[9]);
        a.seed = (uint32_t)strtoul(argv[10], nullptr, 10);
        a.record_dag = 1;
        a.dag_prefix = argv[11];
        std::vector<int> bs(a.num_blocks);
        orc::block_sizes(a.block_size, a.num_blocks, a.upper_block_size, bs.data());
        long N = 0;
        for (int b : bs) N += b;
        std::vector<double> L;
        orc_chol_out o{};
        if (argc >= 13) {
            L.resize((size_t)N * N);
            o.L = L.data();
        }
        int r = orc::cholesky_run<ttor::Threadpool_shared, RefFlow>(&a, &o);
        if (r != 0) return 1;
        if (argc >= 13) {
            FILE* f = fopen(argv[12], "wb");
            fwrite(L.data(), sizeof(double), L.size(), f);
            fclose(f);
        }
        printf("tasks_run %ld edges %ld errors %ld info %d time %e blas %s\n", o.n_tasks_run, o.n_edges, o.errors, o.info,
               o.time_s, o.blas);
        return o.errors ? 1 : 0;
    }
    if (what == "gemm" && argc >= 8) {
        orc_gemm_args a{};
        a.n_threads = atoi(argv[2]);
        a.matrix_size = atoi(argv[3]);
        a.block_size = atoi(argv[4]);
        a.inputs = atoi(argv[5]);
        a.seed = (uint32_t)strtoul(argv[6], nullptr, 10);
        a.record_dag = 1;
        a.dag_prefix = argv[7];
        std::vector<double> C;
        orc_gemm_out o{};
        if (argc >= 9) {
            C.resize((size_t)a.matrix_size * a.matrix_size);
            o.C = C.data();
        }
        int r = orc::gemm_run<ttor::Threadpool_shared, RefFlow>(&a, &o);
        if (r != 0) return 1;
        if (argc >= 9) {
            FILE* f = fopen(argv[8], "wb");
            fwrite(C.data(), sizeof(double), C.size(), f);
            fclose(f);
        }
        printf("tasks_run %ld edges %ld errors %ld time %e blas %s\n", o.n_tasks_run, o.n_edges, o.errors, o.time_s, o.blas);
        return o.errors ? 1 : 0;
    }
    fprintf(stderr, "usage: see the header of ref_driver.cpp\n");
    return 2;
}
