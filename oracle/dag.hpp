/*
 * dag.hpp — TEST INFRASTRUCTURE ONLY.  The single-rank task graphs of the
 * reference's miniapps, written once as templates over the runtime
 * (Threadpool, Taskflow<K>) so the same graph runs on the oracle's restated
 * runtime (runtime.hpp, liboracle.so) and on the reference's own runtime
 * compiled from its sources (ref_driver.cpp, oracle/_ref).
 *
 *  - Cholesky: miniapp/dense_cholesky/2d_cholesky.cpp at nprows = npcols = 1:
 *    block sizes (:63-104), thread map (:125-130), matrix val (:133-147),
 *    priorities (:158-204), names (:206-217), potrf (:316-361), trsm
 *    (:398-464), gemm/syrk (:469-551), accu (:556-608), seed (:613-615).
 *  - GEMM: miniapp/gemm/2d_gemm.cpp at one rank: inputs (:31-40,
 *    gemm_shared.hpp:74-76), send_Aij (:98-120), send_Bij (:122-144),
 *    gemm_Cikj (:151-168), seeding (:174-181).
 *
 * A Recorder logs, per task name, the indegree, the promises received and the
 * runs, and one "src,dst" edge per promise ("ROOT" for the main thread) —
 * the format of the reference's DepsLogger (tasktorrent/src/util.cpp:103-115).
 */
#ifndef TTG_ORACLE_DAG_HPP
#define TTG_ORACLE_DAG_HPP

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../include/ttg_philox.h"
#include "oracle_blas.h"

extern "C" {

typedef struct orc_chol_args {
    int n_threads;
    int block_size;
    int num_blocks;
    int prio_kind;        /* --kind: 0 none, 1 row, 2 critical path, 3 cp+row */
    int accumulate;       /* --accumulate */
    int upper_block_size; /* --upper_block_size (-1 = block_size) */
    int matrix;           /* 0: miniapp val(i,j); 1: G·Gᵀ/N + αI */
    double alpha;
    uint32_t seed;
    int record_dag;
    const char* dag_prefix; /* <prefix>.tasks.csv / <prefix>.edges.csv */
    /* Bounded CPU samples of a large factorisation: run only the tasks of
     * the first panel_limit panel steps (potrf j, trsm (i,j) with j < limit,
     * gemm (k,i,j) with k < limit; every predecessor of such a task is one
     * too).  0 = the whole graph. */
    int panel_limit;
    /* matrix 2: the input as packed lower tiles (tile (i,j), i >= j, column
     * of tiles after column of tiles, each column-major with ld = bs[i]). */
    const double* in_tiles;
} orc_chol_args;

typedef struct orc_chol_out {
    double* L;     /* optional N×N column-major (lower; upper zeroed) */
    double* A;     /* optional N×N column-major input (symmetric) */
    double time_s; /* seeding to join */
    double potrf_s, trsm_s, gemm_s, accu_s;
    double flops;  /* of the tasks run: potrf b^3/3, trsm m b^2, syrk b^2 k, gemm 2 m n k */
    long n_tasks_run;
    long n_edges;
    long errors;
    int info;      /* first failing POTRF (0 = ok) */
    char blas[256];
} orc_chol_out;

typedef struct orc_gemm_args {
    int n_threads;
    int matrix_size;
    int block_size;
    int inputs; /* 0: val_global (A = B); 1: iid U[-1,1] (A stream 2, B stream 3) */
    uint32_t seed;
    int record_dag;
    const char* dag_prefix;
} orc_gemm_args;

typedef struct orc_gemm_out {
    double* C; /* optional N×N column-major */
    double time_s;
    long n_tasks_run;
    long n_edges;
    long errors;
    char blas[256];
} orc_gemm_out;
}

namespace orc {

using clk = std::chrono::steady_clock;
typedef std::array<int, 2> K2;
typedef std::array<int, 3> K3;

inline std::string s_(int v) { return std::to_string(v); }

struct Recorder {
    bool on = false;
    std::mutex mtx;
    std::map<std::string, std::array<long, 3>> tasks; /* indegree, promises, runs */
    std::vector<std::pair<std::string, std::string>> edges;

    static std::string& current() {
        static thread_local std::string c = "ROOT";
        return c;
    }
    void begin(const std::string& name) {
        if (!on) return;
        current() = name;
        std::lock_guard<std::mutex> g(mtx);
        tasks[name][2] += 1;
    }
    void end() {
        if (on) current() = "ROOT";
    }
    void promise(const std::string& dst, int indegree) {
        if (!on) return;
        std::lock_guard<std::mutex> g(mtx);
        auto& e = tasks[dst];
        e[0] = indegree;
        e[1] += 1;
        edges.emplace_back(current(), dst);
    }
    long runs() const {
        long r = 0;
        for (auto& kv : tasks) r += kv.second[2];
        return r;
    }
    void write(const char* prefix) {
        if (!prefix || !*prefix) return;
        std::ofstream tf(std::string(prefix) + ".tasks.csv");
        tf << "name,indegree,promises,runs\n";
        for (auto& kv : tasks) tf << kv.first << "," << kv.second[0] << "," << kv.second[1] << "," << kv.second[2] << "\n";
        std::vector<std::pair<std::string, std::string>> e = edges;
        std::sort(e.begin(), e.end());
        std::ofstream ef(std::string(prefix) + ".edges.csv");
        for (auto& p : e) ef << p.first << "," << p.second << "\n";
    }
};

template <class F>
inline void parallel_for(long n, F f) {
    const int nt = (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    std::atomic<long> next(0);
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&] {
            for (long i = next++; i < n; i = next++) f(i);
        });
    for (auto& x : th) x.join();
}

/* Dense symmetric A = G·Gᵀ/N + αI, G the quantised Gaussian of ttg_philox.h:
 * exact integer dot products, one IEEE division, one addition on the
 * diagonal. */
inline void gen_gram(int N, double alpha, uint32_t seed, double* A) {
    std::vector<int8_t> G((size_t)N * N);
    const size_t total = (size_t)N * N, pairs = (total + 1) / 2;
    parallel_for((long)((pairs + 4095) / 4096), [&](long blk) {
        for (size_t p = (size_t)blk * 4096; p < std::min(pairs, (size_t)(blk + 1) * 4096); ++p) {
            double z[2];
            ttg_normal2(p, seed, TTG_STREAM_G, &z[0], &z[1]);
            for (int h = 0; h < 2; ++h) {
                const size_t e = 2 * p + h;
                if (e >= total) break;
                double t = z[h] * 16.0;
                if (t > 127.0) t = 127.0;
                if (t < -127.0) t = -127.0;
                G[e] = (int8_t)(int)rint(t);
            }
        }
    });
    std::vector<int8_t> Gr(total); /* row-major copy */
    for (int k = 0; k < N; ++k)
        for (int i = 0; i < N; ++i) Gr[(size_t)i * N + k] = G[i + (size_t)k * N];
    const double scale = 256.0 * (double)N;
    parallel_for(N, [&](long j) {
        const int8_t* gj = &Gr[(size_t)j * N];
        for (int i = (int)j; i < N; ++i) {
            const int8_t* gi = &Gr[(size_t)i * N];
            int64_t s = 0;
            for (int k = 0; k < N; ++k) s += (int32_t)gi[k] * (int32_t)gj[k];
            double v = (double)s / scale;
            if (i == j) v = v + alpha;
            A[i + (size_t)j * N] = v;
            A[j + (size_t)i * N] = v;
        }
    });
}

/* Block sizes as 2d_cholesky.cpp:63-104: uniform unless upper > block. */
inline int block_sizes(int block_size, int num_blocks, int upper, int* sizes) {
    const int N = block_size * num_blocks;
    if (upper < 0) upper = block_size;
    if (upper < block_size || upper > 2 * block_size) return -1;
    const int lower = 2 * block_size - upper;
    std::mt19937 gen(2020);
    std::uniform_int_distribution<> distrib(lower, upper);
    int n = 0;
    for (int i = 0; i < num_blocks; ++i) sizes[i] = block_size;
    for (int i = 0; i < num_blocks - 1; ++i) {
        const int bs = std::min(N - n, distrib(gen));
        n += bs;
        sizes[i] = bs;
    }
    sizes[num_blocks - 1] = N - n;
    return 0;
}

inline double val_global(int i, int j) { return (double)((i % 49) + (j % 37) * 53); }

/* The Cholesky task graph at one rank on runtime (Pool, Flow). */
template <class Pool, template <class> class Flow>
int cholesky_run(const orc_chol_args* a, orc_chol_out* out) {
    const int nb = a->num_blocks, n_threads = a->n_threads;
    const int ub = a->upper_block_size < 0 ? a->block_size : a->upper_block_size;
    std::vector<int> bs(nb);
    if (block_sizes(a->block_size, nb, ub, bs.data()) != 0) return -1;
    std::vector<int> displ(nb + 1, 0);
    for (int i = 0; i < nb; ++i) displ[i + 1] = displ[i] + bs[i];
    const int N = displ[nb];
    const bool accumulate = a->accumulate != 0;

    std::vector<double> Ad;
    if (a->matrix == 1) {
        Ad.resize((size_t)N * N);
        gen_gram(N, a->alpha, a->seed, Ad.data());
    }
    if (a->matrix == 2 && !a->in_tiles) return -1;
    auto val = [&](int i, int j) -> double {
        if (a->matrix == 1) return Ad[i + (size_t)j * N];
        return 1.0 / (double)((i - j) * (i - j) + 1);
    };
    std::vector<std::vector<double>> blocks((size_t)nb * nb);
    size_t packed = 0;  // matrix 2: offset of tile (ii, jj) in the packed input
    for (int jj = 0; jj < nb; ++jj)
        for (int ii = jj; ii < nb; ++ii) {
            auto& t = blocks[ii + (size_t)jj * nb];
            t.resize((size_t)bs[ii] * bs[jj]);
            if (a->matrix == 2) {
                std::copy(a->in_tiles + packed, a->in_tiles + packed + t.size(), t.begin());
                packed += t.size();
                continue;
            }
            for (int j = 0; j < bs[jj]; ++j)
                for (int i = 0; i < bs[ii]; ++i) t[i + (size_t)j * bs[ii]] = val(displ[ii] + i, displ[jj] + j);
        }
    if (out->A && a->matrix == 2) {
        for (int jj = 0; jj < nb; ++jj)
            for (int ii = jj; ii < nb; ++ii) {
                const auto& t = blocks[ii + (size_t)jj * nb];
                for (int j = 0; j < bs[jj]; ++j)
                    for (int i = 0; i < bs[ii]; ++i) {
                        const double v = t[i + (size_t)j * bs[ii]];
                        out->A[displ[ii] + i + (size_t)(displ[jj] + j) * N] = v;
                        out->A[displ[jj] + j + (size_t)(displ[ii] + i) * N] = v;
                    }
            }
    } else if (out->A)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) out->A[i + (size_t)j * N] = val(i, j);
    Ad.clear();
    Ad.shrink_to_fit();

    auto lda = [&](int i) { return std::max(1, bs[i]); };
    auto block_2_thread = [&](int i, int j) { return (i + j * nb) % n_threads; };
    const int pk = a->prio_kind;
    auto potf_prio = [&](int j) -> double {
        if (pk == 3) return (double)(9 * (nb - j) - 1) + 18 * nb * nb;
        if (pk == 2) return (double)(9 * (nb - j) - 1);
        if (pk == 1) return 3.0 * (double)(nb - j);
        return 3.0;
    };
    auto trsm_prio = [&](K2 ij) -> double {
        if (pk == 3) return (double)((nb - ij[0]) + nb * (9.0 * nb - 9.0 * ij[1] - 2.0) + 9 * nb * nb);
        if (pk == 2) return (double)(9 * (nb - ij[1]) - 2);
        if (pk == 1) return 2.0 * (double)(nb - ij[0]);
        return 2.0;
    };
    auto gemm_prio = [&](K3 kij) -> double {
        if (pk == 3) {
            if (accumulate) return (double)(nb - kij[1]) + nb * (9.0 * nb - 9.0 * kij[2] - 2.0);
            return (double)(nb - kij[1]) + nb * (9.0 * nb - 3.0 * kij[2] - 6.0 * kij[0] - 2.0);
        }
        if (pk == 2) return (double)(9 * nb - 9 * kij[2] - 2);
        if (pk == 1) return (double)(nb - kij[1]);
        return 1.0;
    };
    auto potrf_name = [](int j) { return "POTRF_" + s_(j); };
    auto trsm_name = [](K2 ij) { return "TRSM_" + s_(ij[0]) + "_" + s_(ij[1]); };
    auto gemm_name = [](K3 kij) { return "GEMM_" + s_(kij[0]) + "_" + s_(kij[1]) + "_" + s_(kij[2]); };
    auto accu_name = [](K3 kij) { return "ACCU_" + s_(kij[0]) + "_" + s_(kij[1]) + "_" + s_(kij[2]); };
    auto potrf_indeg = [&](int j) { return accumulate ? (j == 0 ? 1 : j) : 1; };
    auto trsm_indeg = [&](K2 ij) { return accumulate ? 1 + ij[1] : 1 + (ij[1] == 0 ? 0 : 1); };
    auto gemm_indeg = [&](K3 kij) {
        if (accumulate) return kij[1] == kij[2] ? 1 : 2;
        return (kij[1] == kij[2] ? 1 : 2) + (kij[0] == 0 ? 0 : 1);
    };

    // Tasks of the first `limit` panel steps only (bounded samples).
    const int limit = a->panel_limit > 0 ? std::min(a->panel_limit, nb) : nb;
    std::atomic<long long> flops_x3(0);  // 3 × flops, exact integers
    std::atomic<long> ran(0);            // task bodies run

    Recorder rec;
    rec.on = a->record_dag != 0;
    std::atomic<long long> t_potrf(0), t_trsm(0), t_gemm(0), t_accu(0);
    std::atomic<int> info(0);
    struct Acc {
        std::mutex m;
        std::map<int, std::vector<double>> parts;
    };
    std::vector<Acc> acc((size_t)nb * nb);
    auto us = [](clk::time_point s) {
        return (long long)std::chrono::duration_cast<std::chrono::microseconds>(clk::now() - s).count();
    };

    Pool tp(n_threads, 0, "Wk_Chol_0_");
    Flow<int> potrf(&tp, 0);
    Flow<K2> trsm(&tp, 0);
    Flow<K3> gemm(&tp, 0);
    Flow<K3> accu(&tp, 0);
    auto promise_potrf = [&](int j) {
        if (j >= limit) return;
        rec.promise(potrf_name(j), potrf_indeg(j));
        potrf.fulfill_promise(j);
    };
    auto promise_trsm = [&](K2 ij) {
        if (ij[1] >= limit) return;
        rec.promise(trsm_name(ij), trsm_indeg(ij));
        trsm.fulfill_promise(ij);
    };
    auto promise_gemm = [&](K3 kij) {
        if (kij[0] >= limit) return;
        rec.promise(gemm_name(kij), gemm_indeg(kij));
        gemm.fulfill_promise(kij);
    };
    auto promise_accu = [&](K3 kij) { rec.promise(accu_name(kij), 1); accu.fulfill_promise(kij); };

    potrf.set_task([&](int j) {
             rec.begin(potrf_name(j));
             auto s = clk::now();
             const int r = dpotrf_l(bs[j], blocks[j + (size_t)j * nb].data(), lda(j));
             flops_x3 += (long long)bs[j] * bs[j] * bs[j];
             ++ran;
             if (r != 0) {
                 int z = 0;
                 info.compare_exchange_strong(z, displ[j] + r);
             }
             t_potrf += us(s);
         })
        .set_fulfill([&](int j) {
            for (int i = j + 1; i < nb; ++i) promise_trsm({i, j});
            rec.end();
        })
        .set_indegree(potrf_indeg)
        .set_priority(potf_prio)
        .set_mapping([&](int j) { return block_2_thread(j, j); })
        .set_name(potrf_name);

    trsm.set_task([&](K2 ij) {
            rec.begin(trsm_name(ij));
            auto s = clk::now();
            const int i = ij[0], j = ij[1];
            dtrsm_rltn(bs[i], bs[j], 1.0, blocks[j + (size_t)j * nb].data(), lda(j), blocks[i + (size_t)j * nb].data(), lda(i));
            flops_x3 += 3LL * bs[i] * bs[j] * bs[j];
            ++ran;
            t_trsm += us(s);
        })
        .set_fulfill([&](K2 ij) {
            const int i = ij[0], j = ij[1];
            for (int k = j + 1; k < i; ++k) promise_gemm({j, i, k});
            for (int k = i; k < nb; ++k) promise_gemm({j, k, i});
            rec.end();
        })
        .set_indegree(trsm_indeg)
        .set_priority(trsm_prio)
        .set_mapping([&](K2 ij) { return block_2_thread(ij[0], ij[1]); })
        .set_name(trsm_name);

    gemm.set_task([&](K3 kij) {
            rec.begin(gemm_name(kij));
            auto s = clk::now();
            const int k = kij[0], i = kij[1], j = kij[2];
            std::vector<double> tmp;
            double* C = blocks[i + (size_t)j * nb].data();
            double beta = 1.0;
            if (accumulate) {
                tmp.assign((size_t)bs[i] * bs[j], 0.0);
                C = tmp.data();
                beta = 0.0;
            }
            if (i == j)
                dsyrk_ln(bs[i], bs[k], -1.0, blocks[i + (size_t)k * nb].data(), lda(i), beta, C, lda(i));
            else
                dgemm(NoTrans, Trans, bs[i], bs[j], bs[k], -1.0, blocks[i + (size_t)k * nb].data(), lda(i),
                      blocks[j + (size_t)k * nb].data(), lda(j), beta, C, lda(i));
            flops_x3 += (i == j ? 3LL : 6LL) * bs[i] * bs[j] * bs[k];
            ++ran;
            t_gemm += us(s);
            if (accumulate) {
                std::lock_guard<std::mutex> g(acc[i + (size_t)j * nb].m);
                acc[i + (size_t)j * nb].parts[k] = std::move(tmp);
            }
        })
        .set_fulfill([&](K3 kij) {
            const int k = kij[0], i = kij[1], j = kij[2];
            if (accumulate) promise_accu(kij);
            else if (k < j - 1) promise_gemm({k + 1, i, j});
            else if (i == j) promise_potrf(i);
            else promise_trsm({i, j});
            rec.end();
        })
        .set_indegree(gemm_indeg)
        .set_priority(gemm_prio)
        .set_mapping([&](K3 kij) { return block_2_thread(kij[1], kij[2]); })
        .set_binding([](K3) { return 0; })
        .set_name(gemm_name);

    accu.set_task([&](K3 kij) {
            rec.begin(accu_name(kij));
            auto s = clk::now();
            const int k = kij[0], i = kij[1], j = kij[2];
            std::vector<double> part;
            {
                std::lock_guard<std::mutex> g(acc[i + (size_t)j * nb].m);
                part = std::move(acc[i + (size_t)j * nb].parts[k]);
                acc[i + (size_t)j * nb].parts.erase(k);
            }
            auto& C = blocks[i + (size_t)j * nb];
            for (size_t e = 0; e < C.size(); ++e) C[e] += part[e];
            t_accu += us(s);
            ++ran;
        })
        .set_fulfill([&](K3 kij) {
            if (kij[1] == kij[2]) promise_potrf(kij[1]);
            else promise_trsm({kij[1], kij[2]});
            rec.end();
        })
        .set_indegree([](K3) { return 1; })
        .set_mapping([&](K3 kij) { return block_2_thread(kij[1], kij[2]); })
        .set_priority(gemm_prio)
        .set_binding([](K3) { return 1; })
        .set_name(accu_name);

    auto t0 = clk::now();
    promise_potrf(0);
    tp.join();
    out->time_s = std::chrono::duration<double>(clk::now() - t0).count();
    out->potrf_s = t_potrf.load() * 1e-6;
    out->trsm_s = t_trsm.load() * 1e-6;
    out->gemm_s = t_gemm.load() * 1e-6;
    out->accu_s = t_accu.load() * 1e-6;
    out->flops = (double)flops_x3.load() / 3.0;
    out->info = info.load();
    out->errors = 0;
    for (auto& kv : rec.tasks)
        if (kv.second[1] > kv.second[0] || kv.second[2] != 1) out->errors++;
    out->n_tasks_run = rec.on ? rec.runs() : ran.load();
    out->n_edges = (long)rec.edges.size();
    snprintf(out->blas, sizeof(out->blas), "%s", blas().name.c_str());
    if (out->L) {
        for (size_t e = 0; e < (size_t)N * N; ++e) out->L[e] = 0.0;
        for (int ii = 0; ii < nb; ++ii)
            for (int jj = 0; jj <= ii; ++jj) {
                auto& t = blocks[ii + (size_t)jj * nb];
                for (int j = 0; j < bs[jj]; ++j)
                    for (int i = 0; i < bs[ii]; ++i) {
                        if (ii == jj && i < j) continue;
                        out->L[displ[ii] + i + (size_t)(displ[jj] + j) * N] = t[i + (size_t)j * bs[ii]];
                    }
            }
    }
    if (rec.on) rec.write(a->dag_prefix);
    return 0;
}

/* The 2D block GEMM task graph at one rank on runtime (Pool, Flow). */
template <class Pool, template <class> class Flow>
int gemm_run(const orc_gemm_args* a, orc_gemm_out* out) {
    const int N = a->matrix_size, b = a->block_size;
    if (b <= 0 || N % b != 0) return -1;
    const int nb = N / b, n_threads = a->n_threads;
    std::vector<std::vector<double>> A((size_t)nb * nb), B((size_t)nb * nb), C((size_t)nb * nb);
    for (int bi = 0; bi < nb; ++bi)
        for (int bj = 0; bj < nb; ++bj) {
            auto& ta = A[bi + (size_t)bj * nb];
            auto& tb = B[bi + (size_t)bj * nb];
            ta.resize((size_t)b * b);
            tb.resize((size_t)b * b);
            C[bi + (size_t)bj * nb].assign((size_t)b * b, 0.0);
            for (int j = 0; j < b; ++j)
                for (int i = 0; i < b; ++i) {
                    const int gi = bi * b + i, gj = bj * b + j;
                    const size_t e = gi + (size_t)gj * N;
                    if (a->inputs == 0) {
                        ta[i + (size_t)j * b] = val_global(gi, gj);
                        tb[i + (size_t)j * b] = val_global(gi, gj);
                    } else {
                        ta[i + (size_t)j * b] = ttg_uniform_pm1_at(e, a->seed, TTG_STREAM_GEMM_A);
                        tb[i + (size_t)j * b] = ttg_uniform_pm1_at(e, a->seed, TTG_STREAM_GEMM_B);
                    }
                }
        }
    auto sendA_name = [](K2 ij) { return "send_A_" + s_(ij[0]) + "_" + s_(ij[1]); };
    auto sendB_name = [](K2 ij) { return "send_B_" + s_(ij[0]) + "_" + s_(ij[1]); };
    auto prod_name = [](K3 ikj) { return "prod_C_" + s_(ikj[0]) + "_" + s_(ikj[1]) + "_" + s_(ikj[2]); };
    auto prod_indeg = [](K3 ikj) { return ikj[1] == 0 ? 2 : 3; };
    Recorder rec;
    rec.on = a->record_dag != 0;
    Pool tp(n_threads, 0, "Wk_Gemm_0_");
    Flow<K2> send_A(&tp, 0), send_B(&tp, 0);
    Flow<K3> prod(&tp, 0);
    auto promise_prod = [&](K3 k) { rec.promise(prod_name(k), prod_indeg(k)); prod.fulfill_promise(k); };

    send_A.set_task([&](K2 ij) {
              rec.begin(sendA_name(ij));
              for (int k = 0; k < nb; ++k) promise_prod({ij[0], ij[1], k});
              rec.end();
          })
        .set_indegree([](K2) { return 1; })
        .set_priority([&](K2 ij) { return (double)(nb - ij[1]); })
        .set_mapping([&](K2 ij) { return (ij[0] + ij[1] * nb) % n_threads; })
        .set_name(sendA_name);
    send_B.set_task([&](K2 ij) {
              rec.begin(sendB_name(ij));
              for (int k = 0; k < nb; ++k) promise_prod({k, ij[0], ij[1]});
              rec.end();
          })
        .set_indegree([](K2) { return 1; })
        .set_priority([&](K2 ij) { return (double)(nb - ij[0]); })
        .set_mapping([&](K2 ij) { return (ij[0] + ij[1] * nb) % n_threads; })
        .set_name(sendB_name);
    prod.set_task([&](K3 ikj) {
            rec.begin(prod_name(ikj));
            const int i = ikj[0], k = ikj[1], j = ikj[2];
            dgemm(NoTrans, NoTrans, b, b, b, 1.0, A[i + (size_t)k * nb].data(), b, B[k + (size_t)j * nb].data(), b, 1.0,
                  C[i + (size_t)j * nb].data(), b);
            if (k < nb - 1) promise_prod({i, k + 1, j});
            rec.end();
        })
        .set_indegree(prod_indeg)
        .set_mapping([&](K3 ikj) { return (ikj[0] + ikj[2] * nb) % n_threads; })
        .set_name(prod_name);

    auto t0 = clk::now();
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) {
            rec.promise(sendA_name({i, j}), 1);
            send_A.fulfill_promise({i, j});
            rec.promise(sendB_name({i, j}), 1);
            send_B.fulfill_promise({i, j});
        }
    tp.join();
    out->time_s = std::chrono::duration<double>(clk::now() - t0).count();
    out->n_tasks_run = rec.runs();
    out->n_edges = (long)rec.edges.size();
    out->errors = 0;
    for (auto& kv : rec.tasks)
        if (kv.second[1] > kv.second[0] || kv.second[2] != 1) out->errors++;
    snprintf(out->blas, sizeof(out->blas), "%s", blas().name.c_str());
    if (out->C) {
        for (int bi = 0; bi < nb; ++bi)
            for (int bj = 0; bj < nb; ++bj)
                for (int j = 0; j < b; ++j)
                    for (int i = 0; i < b; ++i)
                        out->C[bi * b + i + (size_t)(bj * b + j) * N] = C[bi + (size_t)bj * nb][i + (size_t)j * b];
    }
    if (rec.on) rec.write(a->dag_prefix);
    return 0;
}

}  // namespace orc

#endif
