// 2d_cholesky — the reference's dense Cholesky miniapp command line
// (miniapp/dense_cholesky/2d_cholesky.cpp:692-752) on the GB300 executor.
//
// Same flags and defaults; one rank only (--nprows/--npcols other than 1 are
// rejected: there is no MPI in this build).  --n_threads is the task graph's
// mapping modulus (the reference's thread count); the device runs the graph
// with one persistent block per SM unless --workers says otherwise.
// Additions: --matrix (miniapp | gram), --alpha, --seed, --precision
// (fp64 | mixed), --workers, --reps, --dag (DAG record prefix).
// Output keeps the reference's lines: "Elapsed time", the per-kind times,
// the ">>>>" summary and "=> Error solve" of --test (fails above 1e-6).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <vector>

#include "../../include/ttg.h"
#include "../../include/ttg_apps.h"
#include "args.hpp"

static int fail(const char* what, ttg_status s) {
    fprintf(stderr, "2d_cholesky: %s: %s\n", what, ttg_strerror(s));
    return 1;
}

int main(int argc, const char** argv) {
    Args args("2d_cholesky", "2D dense cholesky using TaskTorrent (GB300 executor)");
    args.add("n_threads", "Number of threads (mapping modulus)", "2");
    args.add("verb", "Verbosity level", "0");
    args.add("block_size", "Block size", "5");
    args.add("num_blocks", "Number of blocks", "10");
    args.add("nprows", "Number of processors accross rows", "1");
    args.add("npcols", "Number of processors accross columns", "1");
    args.add("kind", "Priority kind", "0");
    args.add("log", "Enable logging", "false");
    args.add("depslog", "Enable dependency logging", "false");
    args.add("test", "Test or not", "true");
    args.add("accumulate", "Accumulate block GEMMs in parallel", "false");
    args.add("upper_block_size", "Upper block size", "-1");
    args.add("matrix", "Input matrix: miniapp (1/((i-j)^2+1)) or gram (G*G^T/N + alpha*I)", "miniapp");
    args.add("alpha", "Diagonal shift of the gram matrix", "1.0");
    args.add("seed", "Seed of the gram matrix", "0");
    args.add("precision", "fp64 or mixed", "fp64");
    args.add("workers", "Persistent blocks (0 = one per SM)", "0");
    args.add("reps", "Timed repetitions", "1");
    try {
        args.parse(argc, argv);
    } catch (const std::exception& e) {
        fprintf(stderr, "2d_cholesky: %s\n", e.what());
        return 2;
    }
    if (args.help) {
        args.print_help();
        return 0;
    }
    const int block_size = args.i("block_size"), num_blocks = args.i("num_blocks"), n_threads = args.i("n_threads");
    const int upper = args.i("upper_block_size") == -1 ? block_size : args.i("upper_block_size");
    if (args.i("nprows") != 1 || args.i("npcols") != 1) {
        fprintf(stderr, "2d_cholesky: this build runs one rank (nprows = npcols = 1)\n");
        return 2;
    }
    if (block_size <= 0 || num_blocks <= 0 || n_threads <= 0 || upper < block_size || upper > 2 * block_size) {
        fprintf(stderr, "2d_cholesky: invalid sizes\n");
        return 2;
    }
    const bool log = args.b("log"), depslog = args.b("depslog"), test = args.b("test");
    printf("Arguments: block_size (size of blocks) %d\nnum_blocks (# of blocks) %d\nn_threads %d\nverb %d\nnprows 1\nnpcols 1\n"
           "kind %d\nlog %d\ndeplog %d\ntest %d\naccumulate %d\nupper_block_size %d\n",
           block_size, num_blocks, n_threads, args.i("verb"), args.i("kind"), log, depslog, test, (int)args.b("accumulate"), upper);

    ttg_opts o{};
    o.workers = args.i("workers");
    o.timeout_s = 60.0;
    o.trace = 1;
    ttg_ctx* ctx = nullptr;
    ttg_status s = ttg_create(&ctx, &o);
    if (s != TTG_OK) return fail("ttg_create", s);

    ttg_chol_args ca{};
    ca.n_threads = n_threads;
    ca.verb = args.i("verb");
    ca.block_size = block_size;
    ca.num_blocks = num_blocks;
    ca.kind = args.i("kind");
    ca.accumulate = args.b("accumulate");
    ca.upper_block_size = upper;
    ca.matrix = args.s("matrix") == "gram" ? 1 : 0;
    ca.alpha = args.d("alpha");
    ca.seed = (uint32_t)args.i("seed");
    ca.precision = args.s("precision") == "mixed" ? TTG_PREC_MIXED : TTG_PREC_F64;
    ttg_chol_plan* plan = nullptr;
    s = ttg_chol_plan_create(ctx, &ca, &plan);
    if (s != TTG_OK) return fail("plan", s);
    std::vector<int32_t> bs(num_blocks);
    const int N = ttg_chol_plan_n(plan, bs.data());
    printf("lower_block_size %d, upper_block_size %d\nblock sizes: ", 2 * block_size - upper, upper);
    for (int b : bs) printf("%d ", b);
    printf("\n");
    double capture_s = 0;
    const int ntasks = ttg_chol_plan_tasks(plan, &capture_s);

    printf("Starting Cholesky factorization...\n");
    double best_ms = 1e30;
    ttg_report rep{};
    for (int r = 0; r < std::max(1, args.i("reps")); ++r) {
        ttg_chol_plan_restore(plan, nullptr);
        s = ttg_chol_plan_factor(plan, nullptr, &rep);
        if (s != TTG_OK) return fail("factor", s);
        best_ms = std::min(best_ms, (double)rep.elapsed_ms);
    }
    const double total_time = best_ms * 1e-3;
    double tp = 0, tt = 0, tg = 0, ta = 0;
    ttg_chol_plan_kind_times(plan, &tp, &tt, &tg, &ta);
    printf("Done with Cholesky factorization...\n");
    printf("Elapsed time: %e\n", total_time);
    printf("Potrf time: %e\n", tp * 1e-3);
    printf("Trsm time: %e\n", tt * 1e-3);
    printf("Gemm time: %e\n", tg * 1e-3);
    printf("Accu time: %e\n", ta * 1e-3);
    printf("Capture time: %e (%d device tasks, %d workers)\n", capture_s, ntasks, rep.workers);
    printf("++++rank nranks n_threads matrix_size block_size num_blocks priority_kind accumulate upper_block_size total_time\n");
    printf("[0]>>>>0 1 %d %d %d %d %d %d %d %e\n", n_threads, N, block_size, num_blocks, ca.kind, ca.accumulate, upper, total_time);
    printf("GFLOP/s (N^3/3): %.3f\n", (double)N * N * N / 3.0 / total_time * 1e-9);

    if (log || depslog) {
        // The reference's file names (2d_cholesky.cpp:630-644) at one rank.
        const std::string base = "ttor_dist_" + std::to_string(block_size) + "_" + std::to_string(num_blocks) + "_1_" +
                                 std::to_string(n_threads) + "_" + std::to_string(ca.kind);
        const std::string logname = base + ".log.0", depsname = "deps_" + base + ".dot.0";
        s = ttg_chol_plan_write_log(plan, log ? logname.c_str() : nullptr, depslog ? depsname.c_str() : nullptr);
        if (s != TTG_OK) return fail("write_log", s);
    }

    int rc = 0;
    if (test) {
        printf("Starting test on rank 0...\n");
        std::vector<double> A((size_t)N * N), L((size_t)N * N);
        ttg_chol_plan_get_input(plan, A.data());
        ttg_chol_plan_get_factor(plan, L.data());
        std::mt19937 gen(2019);
        std::uniform_real_distribution<double> dist(-1.0, 1.0);
        std::vector<double> x(N), b(N, 0.0);
        for (auto& v : x) v = dist(gen);
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) b[i] += A[i + (size_t)j * N] * x[j];
        for (int j = 0; j < N; ++j) {  // L y = b
            b[j] /= L[j + (size_t)j * N];
            for (int i = j + 1; i < N; ++i) b[i] -= L[i + (size_t)j * N] * b[j];
        }
        for (int j = N - 1; j >= 0; --j) {  // Lᵀ x = y
            double v = b[j];
            for (int i = j + 1; i < N; ++i) v -= L[i + (size_t)j * N] * b[i];
            b[j] = v / L[j + (size_t)j * N];
        }
        double num = 0, den = 0;
        for (int i = 0; i < N; ++i) {
            num += (b[i] - x[i]) * (b[i] - x[i]);
            den += x[i] * x[i];
        }
        const double error = std::sqrt(num / den);
        printf("\n=> Error solve %e\n\n", error);
        if (!(error <= 1e-6)) {
            printf("\n\nERROR: error is too large!\n\n");
            rc = 1;
        }
    }
    ttg_chol_plan_destroy(plan);
    ttg_destroy(ctx);
    return rc;
}
