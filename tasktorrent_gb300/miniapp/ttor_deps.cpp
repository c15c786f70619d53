// ttor_deps — the reference's dependency-chain scheduler micro-benchmark
// (miniapp/mini_benchmarks/shared/ttor_deps.cpp) on the GB300 executor:
// n_rows rows of tasks over n_cols columns, task (i, j) fulfilling
// ((i + k) % n_rows, j + 1) for 0 <= k < n_edges from inside its body, each
// keeping its block busy for spin_time seconds.  Same positional arguments
// and defaults: n_threads n_rows n_edges n_cols spin_time repeat verb.
#include <array>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "../tasktorrent/tasktorrent.hpp"
#include "bench_common.hpp"

int main(int argc, char** argv) {
    int n_threads = 1, n_rows = 10, n_edges = 10, n_cols = 5, repeat = 1, verb = 0;
    double spin_time = 1e-6;
    if (argc >= 2 && (n_threads = atoi(argv[1])) <= 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 3 && (n_rows = atoi(argv[2])) <= 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 4 && (n_edges = atoi(argv[3])) <= 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 5 && (n_cols = atoi(argv[4])) <= 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 6 && ((spin_time = atof(argv[5])) < 0 || spin_time > 1.0)) { printf("Wrong argument\n"); return 1; }
    if (argc >= 7 && (repeat = atoi(argv[6])) <= 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 8 && (verb = atoi(argv[7])) < 0) { printf("Wrong argument\n"); return 1; }
    if (verb) printf("./ttor_deps n_threads n_rows n_edges n_cols spin_time repeat verb\n");

    using Key2 = std::array<int, 2>;
    const int n_tasks = n_rows * n_cols;
    ttg_ctx* ctx = ttor::gpu::default_context();
    RepeatStats st;
    int workers = 1;
    for (int step = 0; step < repeat; ++step) {
        ttor::Threadpool_shared tp(n_threads, 0, "Wk_");
        tp.set_context(ctx);
        ttor::Taskflow<Key2> tf(&tp, 0);
        tf.set_mapping([&](Key2 ij) { return ij[0] % n_threads; })
            .set_indegree([&](Key2 ij) { return ij[1] == 0 ? 1 : n_edges; })
            .set_task([&](Key2 ij) {
                ttor::gpu::spin_for_seconds(spin_time);
                if (ij[1] < n_cols - 1)
                    for (int k = 0; k < n_edges; k++) tf.fulfill_promise({(ij[0] + k) % n_rows, ij[1] + 1});
            })
            .set_priority([&](Key2 ij) { return n_cols - (double)ij[1]; })
            .set_name([](Key2 ij) { return std::to_string(ij[0]) + "_" + std::to_string(ij[1]); });
        const auto t0 = ttor::wctime();
        for (int k = 0; k < n_rows; k++) tf.fulfill_promise({k, 0});
        tp.join();
        const double time = ttor::elapsed(t0, ttor::wctime());
        const ttg_report& rep = tp.report();
        if (rep.status != TTG_OK || rep.tasks_run != n_tasks) {
            printf("Error: %s, %lld of %d tasks ran\n", ttg_strerror(rep.status), (long long)rep.tasks_run, n_tasks);
            return 1;
        }
        workers = ttg_workers(ctx);
        const double eff = (double)n_tasks * spin_time / time / (double)workers;
        const double dev_s = rep.elapsed_ms * 1e-3;
        const double dev_eff = dev_s > 0 ? (double)n_tasks * spin_time / dev_s / (double)workers : 0.0;
        if (verb) printf("iteration repeat n_threads n_rows n_edges n_cols spin_time time n_tasks efficiency\n");
        printf("++++ ttor_deps %d %d %d %d %d %d %e %e %d %e\n", step, repeat, workers, n_rows, n_edges, n_cols, spin_time, time, n_tasks,
               eff);
        printf("#### ttor_deps device_time %e device_efficiency %e\n", dev_s, dev_eff);
        st.add(time, eff);
    }
    double em, es, tm, ts;
    RepeatStats::mean_std(st.effs, &em, &es);
    RepeatStats::mean_std(st.times, &tm, &ts);
    printf("]]]] exp repeat n_threads n_rows n_edges n_cols spin_time n_tasks efficiency_mean efficiency_std time_mean time_std\n");
    printf(">>>> ttor_deps %d %d %d %d %d %e %d %e %e %e %e\n", repeat, workers, n_rows, n_edges, n_cols, spin_time, n_tasks, em, es, tm,
           ts);
    return 0;
}
