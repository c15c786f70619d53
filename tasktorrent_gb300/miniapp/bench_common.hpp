// Output of the scheduler micro-benchmarks: the reference's lines
// (miniapp/mini_benchmarks/common.hpp:51-122): one "++++" line per repetition,
// then "]]]]" (column names) and ">>>>" (means and standard deviations).
//
// On the GB300 executor the parallel resources are the persistent blocks,
// so "n_threads" in these lines and the efficiency
//     n_tasks · spin_time / (time · workers)
// use the executor's worker count; the command-line n_threads stays the
// mapping modulus of the task flow, as in the reference.  time is the host
// wall time of the insertion and join() (capture, upload, device run); a
// "####" line per repetition adds the device executor's own time and the
// efficiency measured with it.
#pragma once
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

struct RepeatStats {
    std::vector<double> times, effs;
    void add(double t, double e) {
        times.push_back(t);
        effs.push_back(e);
    }
    static void mean_std(const std::vector<double>& v, double* mean, double* sd) {
        double m = 0.0, s = 0.0;
        for (double x : v) m += x;
        m /= v.empty() ? 1.0 : (double)v.size();
        for (double x : v) s += (x - m) * (x - m);
        *mean = m;
        *sd = v.size() > 1 ? std::sqrt(s / (double)(v.size() - 1)) : 0.0;
    }
};
