// ttor_wait — the reference's "wait only" scheduler micro-benchmark
// (miniapp/mini_benchmarks/shared/ttor_wait.cpp) on the GB300 executor:
// n_tasks independent tasks that each keep their block busy for spin_time
// seconds (ttor::gpu::spin_for_seconds).  Same positional arguments and
// defaults: n_threads n_tasks spin_time time_insertion repeat verb.
// time_insertion = 1 times the insertion (fulfill_promise of every task) and
// join(); 0 times start() and join() only, as in the reference.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "../tasktorrent/tasktorrent.hpp"
#include "bench_common.hpp"

int main(int argc, char** argv) {
    int n_threads = 1, n_tasks = 1000, repeat = 1, verb = 0;
    double spin_time = 1e-6;
    bool time_insertion = true;
    if (argc >= 2 && (n_threads = atoi(argv[1])) <= 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 3 && (n_tasks = atoi(argv[2])) < 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 4 && ((spin_time = atof(argv[3])) < 0 || spin_time > 1.0)) { printf("Wrong argument\n"); return 1; }
    if (argc >= 5) time_insertion = atoi(argv[4]) != 0;
    if (argc >= 6 && (repeat = atoi(argv[5])) <= 0) { printf("Wrong argument\n"); return 1; }
    if (argc >= 7 && (verb = atoi(argv[6])) < 0) { printf("Wrong argument\n"); return 1; }
    if (verb) printf("./ttor_wait n_threads n_tasks spin_time time_insertion repeat verb\n");

    const std::string exp = "ttor_wait_time_insertion" + std::to_string((int)time_insertion);
    ttg_ctx* ctx = ttor::gpu::default_context();
    RepeatStats st;
    int workers = 1;
    for (int step = 0; step < repeat; ++step) {
        ttor::Threadpool_shared tp(n_threads, 0, "Wk_", false);
        tp.set_context(ctx);
        ttor::Taskflow<int> tf(&tp, 0);
        tf.set_mapping([&](int k) { return k % n_threads; })
            .set_indegree([](int) { return 1; })
            .set_task([&](int) { ttor::gpu::spin_for_seconds(spin_time); })
            .set_name([](int k) { return "SPIN_" + std::to_string(k); });
        double time = 0.0;
        if (time_insertion) {
            const auto t0 = ttor::wctime();
            tp.start();
            for (int k = 0; k < n_tasks; k++) tf.fulfill_promise(k);
            tp.join();
            time = ttor::elapsed(t0, ttor::wctime());
        } else {
            for (int k = 0; k < n_tasks; k++) tf.fulfill_promise(k);
            const auto t0 = ttor::wctime();
            tp.start();
            tp.join();
            time = ttor::elapsed(t0, ttor::wctime());
        }
        const ttg_report& rep = tp.report();
        if (rep.status != TTG_OK || rep.tasks_run != n_tasks) {
            printf("Error: %s, %lld of %d tasks ran\n", ttg_strerror(rep.status), (long long)rep.tasks_run, n_tasks);
            return 1;
        }
        workers = ttg_workers(ctx);
        const double eff = (double)n_tasks * spin_time / time / (double)workers;
        const double dev_s = rep.elapsed_ms * 1e-3;
        const double dev_eff = dev_s > 0 ? (double)n_tasks * spin_time / dev_s / (double)workers : 0.0;
        if (verb) printf("iteration repeat n_threads n_tasks spin_time time efficiency\n");
        printf("++++ %s %d %d %d %d %e %e %e\n", exp.c_str(), step, repeat, workers, n_tasks, spin_time, time, eff);
        printf("#### %s device_time %e device_efficiency %e\n", exp.c_str(), dev_s, dev_eff);
        st.add(time, eff);
    }
    double em, es, tm, ts;
    RepeatStats::mean_std(st.effs, &em, &es);
    RepeatStats::mean_std(st.times, &tm, &ts);
    printf("]]]] exp repeat n_threads spin_time n_tasks efficiency_mean efficiency_std time_mean time_std\n");
    printf(">>>> %s %d %d %e %d %e %e %e %e\n", exp.c_str(), repeat, workers, spin_time, n_tasks, em, es, tm, ts);
    return 0;
}
