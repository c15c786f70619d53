// 2d_gemm — the reference's block GEMM miniapp command line
// (miniapp/gemm/2d_gemm.cpp:230-282) on the GB300 executor.
//
// Same flags and defaults; one rank only.  --use_large only selects an MPI
// message kind in the reference and is accepted and ignored.  Additions:
// --inputs (val_global | uniform), --seed, --workers, --reps.  The printed
// FLOP rate uses 2N^3 (the reference's ">>>>" line prints N^3 per rank as its
// "flops" figure, 2d_gemm.cpp:187; that line is kept as is).
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/ttg.h"
#include "../../include/ttg_apps.h"
#include "args.hpp"

int main(int argc, const char** argv) {
    Args args("2d_gemm", "2D dense gemm using TaskTorrent (GB300 executor)");
    args.add("n_threads", "Number of threads (mapping modulus)", "1");
    args.add("verb", "Verbosity level", "0");
    args.add("block_size", "Block size", "8");
    args.add("matrix_size", "Total matrix size", "128");
    args.add("nprows", "Number of processors accross rows", "1");
    args.add("npcols", "Number of processors accross columns", "1");
    args.add("test", "Test or not", "true");
    args.add("use_large", "Use large active messages (ignored: one rank)", "true");
    args.add("inputs", "val_global or uniform", "val_global");
    args.add("seed", "Seed of the uniform inputs", "1");
    args.add("workers", "Persistent blocks (0 = one per SM)", "0");
    args.add("reps", "Timed repetitions", "1");
    try {
        args.parse(argc, argv);
    } catch (const std::exception& e) {
        fprintf(stderr, "2d_gemm: %s\n", e.what());
        return 2;
    }
    if (args.help) {
        args.print_help();
        return 0;
    }
    const int N = args.i("matrix_size"), b = args.i("block_size"), n_threads = args.i("n_threads");
    if (args.i("nprows") != 1 || args.i("npcols") != 1) {
        fprintf(stderr, "2d_gemm: this build runs one rank (nprows = npcols = 1)\n");
        return 2;
    }
    if (b <= 0 || N <= 0 || N % b != 0 || n_threads <= 0) {
        fprintf(stderr, "2d_gemm: matrix_size must be a positive multiple of block_size\n");
        return 2;
    }
    printf("Arguments: block_size %d\nmatrix_size %d\nn_threads %d\nverb %d\nnprows 1\nnpcols 1\ntest %d\nuse_large %d\n", b, N,
           n_threads, args.i("verb"), (int)args.b("test"), (int)args.b("use_large"));
    ttg_opts o{};
    o.workers = args.i("workers");
    o.timeout_s = 60.0;
    ttg_ctx* ctx = nullptr;
    ttg_status s = ttg_create(&ctx, &o);
    if (s != TTG_OK) {
        fprintf(stderr, "2d_gemm: %s\n", ttg_strerror(s));
        return 1;
    }
    ttg_gemm_args ga{};
    ga.n_threads = n_threads;
    ga.verb = args.i("verb");
    ga.block_size = b;
    ga.matrix_size = N;
    ga.inputs = args.s("inputs") == "uniform" ? 1 : 0;
    ga.seed = (uint32_t)args.i("seed");
    ttg_gemm_plan* plan = nullptr;
    s = ttg_gemm_plan_create(ctx, &ga, &plan);
    if (s != TTG_OK) {
        fprintf(stderr, "2d_gemm: plan: %s\n", ttg_strerror(s));
        return 1;
    }
    printf("Starting 2D Gemm...\n");
    double best = 1e30;
    ttg_report rep{};
    for (int r = 0; r < std::max(1, args.i("reps")); ++r) {
        s = ttg_gemm_plan_run(plan, nullptr, &rep);
        if (s != TTG_OK) {
            fprintf(stderr, "2d_gemm: run: %s\n", ttg_strerror(s));
            return 1;
        }
        best = std::min(best, (double)rep.elapsed_ms * 1e-3);
    }
    const long long flops_per_rank = (long long)N * N * N;
    double capture_s = 0;
    ttg_gemm_plan_tasks(plan, &capture_s);
    printf("%e\n", capture_s);
    printf("[rank]>>>>rank n_ranks n_cores nthreads nprows npcols use_large matrix_size num_blocks block_size total_time flops_per_core flops_per_rank\n");
    printf("[0]>>>>ttor_2d_gemm 0 1 %d %d 1 1 %d %d %d %d %e %llu %llu\n", n_threads, n_threads, (int)args.b("use_large"), N, N / b, b,
           best, (unsigned long long)(flops_per_rank / n_threads), (unsigned long long)flops_per_rank);
    printf("GFLOP/s (2N^3): %.3f\n", 2.0 * N * (double)N * N / best * 1e-9);
    int rc = 0;
    if (args.b("test")) {
        printf("Testing..\n");
        std::vector<double> C((size_t)N * N), A((size_t)N * N);
        ttg_gemm_plan_get_C(plan, C.data());
        if (ga.inputs == 0) {
            for (int j = 0; j < N; ++j)
                for (int i = 0; i < N; ++i) A[i + (size_t)j * N] = (double)((i % 49) + (j % 37) * 53);
            double num = 0, den = 0;
            std::vector<double> col(N);
            for (int j = 0; j < N; ++j) {
                std::fill(col.begin(), col.end(), 0.0);
                for (int k = 0; k < N; ++k) {
                    const double bkj = A[k + (size_t)j * N];
                    for (int i = 0; i < N; ++i) col[i] += A[i + (size_t)k * N] * bkj;
                }
                for (int i = 0; i < N; ++i) {
                    const double d = col[i] - C[i + (size_t)j * N];
                    num += d * d;
                    den += col[i] * col[i];
                }
            }
            printf("\n==> GEMM error %e\n\n", std::sqrt(num / den));
        } else {
            printf("(uniform inputs: checked by the test suite against the oracle)\n");
        }
    }
    ttg_gemm_plan_destroy(plan);
    ttg_destroy(ctx);
    return rc;
}
